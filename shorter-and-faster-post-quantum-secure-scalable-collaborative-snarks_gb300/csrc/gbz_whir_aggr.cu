// WHIR aggregation of several claims and commitments (Whir.cpp:547-704):
// inner products of many vector pairs and linear combinations of many
// vectors, each one streaming pass over HBM.
#include "gbz_whir_aggr.cuh"

namespace gbz {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ fe shfl_down_fe(fe v, int d) {
  fe r;
  r.re = __shfl_down_sync(0xffffffffu, v.re, d);
  r.im = __shfl_down_sync(0xffffffffu, v.im, d);
  return r;
}

// out[t] = (acc ? out[t] : 0) + sum_i coef[i] * v.p[i][t]
__global__ void __launch_bounds__(kThreads) lincomb_kernel(VecList v, const fe *coef, int k, uint64_t n, fe *out,
                                                           int acc) {
  __shared__ fe c[kMaxVecs];
  for (int i = threadIdx.x; i < k; i += kThreads) c[i] = coef[i];
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * kThreads;
  for (uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x; t < n; t += stride) {
    fe s = acc ? out[t] : fe_zero();
    for (int i = 0; i < k; i++) s = fadd(s, fmul(c[i], v.p[i][t]));
    out[t] = s;
  }
}

// Per-CTA partial sums of the TA x TB inner products <a_i, b_j>.
template <int TA, int TB>
__global__ void __launch_bounds__(kThreads) multidot_kernel(VecList a, VecList b, uint64_t n, fe *partial) {
  fe acc[TA * TB];
#pragma unroll
  for (int q = 0; q < TA * TB; q++) acc[q] = fe_zero();
  const uint64_t stride = (uint64_t)gridDim.x * kThreads;
  for (uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x; t < n; t += stride) {
    fe x[TA], y[TB];
#pragma unroll
    for (int i = 0; i < TA; i++) x[i] = a.p[i][t];
#pragma unroll
    for (int j = 0; j < TB; j++) y[j] = b.p[j][t];
#pragma unroll
    for (int i = 0; i < TA; i++)
#pragma unroll
      for (int j = 0; j < TB; j++) acc[i * TB + j] = fadd(acc[i * TB + j], fmul(x[i], y[j]));
  }
  __shared__ fe red[TA * TB][kThreads / 32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < TA * TB; q++) {
    fe s = acc[q];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s = fadd(s, shfl_down_fe(s, d));
    if (lane == 0) red[q][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < TA * TB) {
    fe s = fe_zero();
    for (int k = 0; k < kThreads / 32; k++) s = fadd(s, red[threadIdx.x][k]);
    partial[(uint64_t)blockIdx.x * TA * TB + threadIdx.x] = s;
  }
}

// out[q] = sum over blocks of partial[block * nq + q]
__global__ void sum_cols_kernel(const fe *partial, int blocks, int nq, fe *out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  fe s = fe_zero();
  for (int b = 0; b < blocks; b++) s = fadd(s, partial[(uint64_t)b * nq + q]);
  out[q] = s;
}

int grid_for(uint64_t n) {
  uint64_t g = (n + kThreads - 1) / kThreads;
  if (g > 152 * 8) g = 152 * 8;
  return g ? (int)g : 1;
}

template <int TA, int TB>
void md_launch(const VecList &a, const VecList &b, uint64_t n, fe *partial, int blocks, cudaStream_t s) {
  multidot_kernel<TA, TB><<<blocks, kThreads, 0, s>>>(a, b, n, partial);
  GBZ_CUDA(cudaGetLastError());
}

void md_dispatch(int ta, int tb, const VecList &a, const VecList &b, uint64_t n, fe *partial, int blocks,
                 cudaStream_t s) {
#define GBZ_MD(A, B) \
  if (ta == A && tb == B) return md_launch<A, B>(a, b, n, partial, blocks, s);
  GBZ_MD(1, 1) GBZ_MD(1, 2) GBZ_MD(1, 3) GBZ_MD(1, 4)
  GBZ_MD(2, 1) GBZ_MD(2, 2) GBZ_MD(2, 3) GBZ_MD(2, 4)
  GBZ_MD(3, 1) GBZ_MD(3, 2) GBZ_MD(3, 3) GBZ_MD(3, 4)
  GBZ_MD(4, 1) GBZ_MD(4, 2) GBZ_MD(4, 3) GBZ_MD(4, 4)
#undef GBZ_MD
  throw ArgError("multidot: tile out of range");
}

}  // namespace

void lincomb_launch(const VecList &v, const fe *coef, int k, uint64_t n, fe *out, bool accumulate, cudaStream_t s) {
  if (k < 0 || k > kMaxVecs) throw ArgError("linear combination of more than 64 vectors");
  if (!n) return;
  lincomb_kernel<<<grid_for(n), kThreads, 0, s>>>(v, coef, k, n, out, accumulate ? 1 : 0);
  GBZ_CUDA(cudaGetLastError());
}

uint64_t multidot_scratch(uint64_t n) { return (uint64_t)grid_for(n) * 16 + 16; }  // elements

void multidot_launch(const VecList &a, int ka, const VecList &b, int kb, uint64_t n, fe *partial, fe *out,
                     cudaStream_t s) {
  if (ka > kMaxVecs || kb > kMaxVecs) throw ArgError("inner products of more than 64 vectors");
  const int blocks = grid_for(n);
  // 4 x 4 tiles: every tile reads its (up to) 8 vectors once
  for (int i0 = 0; i0 < ka; i0 += 4)
    for (int j0 = 0; j0 < kb; j0 += 4) {
      const int ta = std::min(4, ka - i0), tb = std::min(4, kb - j0);
      VecList at{}, bt{};
      for (int i = 0; i < ta; i++) at.p[i] = a.p[i0 + i];
      for (int j = 0; j < tb; j++) bt.p[j] = b.p[j0 + j];
      md_dispatch(ta, tb, at, bt, n, partial, blocks, s);
      // tile results go to a staging row, then into out[i][j] (row-major ka x kb)
      fe *tile = partial + (uint64_t)blocks * 16;
      sum_cols_kernel<<<1, 32, 0, s>>>(partial, blocks, ta * tb, tile);
      GBZ_CUDA(cudaGetLastError());
      for (int i = 0; i < ta; i++)
        GBZ_CUDA(cudaMemcpyAsync(out + (uint64_t)(i0 + i) * kb + j0, tile + i * tb, sizeof(fe) * tb,
                                 cudaMemcpyDeviceToDevice, s));
    }
}

}  // namespace gbz
