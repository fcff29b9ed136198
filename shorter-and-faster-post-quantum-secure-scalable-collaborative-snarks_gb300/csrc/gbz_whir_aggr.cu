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

// out[q] = sum over blocks of partial[block * nq + q]: one CTA per q
// (launched with nq CTAs of kThreads), the blocks spread over its threads.
__global__ void __launch_bounds__(kThreads) sum_cols_kernel(const fe *partial, int blocks, int nq, fe *out) {
  const int q = blockIdx.x;
  fe s = fe_zero();
  for (int b = threadIdx.x; b < blocks; b += kThreads) s = fadd(s, partial[(uint64_t)b * nq + q]);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) s = fadd(s, shfl_down_fe(s, d));
  __shared__ fe red[kThreads / 32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[w] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    fe t = fe_zero();
    for (int k = 0; k < kThreads / 32; k++) t = fadd(t, red[k]);
    out[q] = t;
  }
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
      sum_cols_kernel<<<ta * tb, kThreads, 0, s>>>(partial, blocks, ta * tb, tile);
      GBZ_CUDA(cudaGetLastError());
      for (int i = 0; i < ta; i++)
        GBZ_CUDA(cudaMemcpyAsync(out + (uint64_t)(i0 + i) * kb + j0, tile + i * tb, sizeof(fe) * tb,
                                 cudaMemcpyDeviceToDevice, s));
    }
}

namespace {

// aggregate_claims by streaming passes (Whir.cpp:608-668): the eq tables
// of the claim points are never written; entry x of table j is elo_j[x mod
// 2^h] times ehi_j[x >> h] (the two halves of the point: the products
// precompute_beta forms, in another order).  One pass takes TC points: it
// reads the TA arrays and forms the TA x TC sums <a_i, eq_j> (per-CTA
// partials), adds sum_j bw[j] eq_j into b_aggr (stores it in the first
// pass) and, when aw is set, stores arr = sum_i aw[i] a_i.  Two points a
// pass keep the accumulators in registers at two CTAs per SM.
template <int TA, int TC>
__global__ void __launch_bounds__(kThreads, 2)
aggr_claims_pass_kernel(VecList a, const fe *elo, const fe *ehi, int h, uint64_t lo_len, uint64_t hi_len,
                        uint64_t n, const fe *bw, const fe *aw, int first, fe *arr, fe *baggr, fe *partial) {
  __shared__ fe sw[TA + TC];
  if (threadIdx.x < TC) sw[threadIdx.x] = bw[threadIdx.x];
  if (aw && threadIdx.x < TA) sw[TC + threadIdx.x] = aw[threadIdx.x];
  __syncthreads();
  fe acc[TA * TC];
#pragma unroll
  for (int q = 0; q < TA * TC; q++) acc[q] = fe_zero();
  const uint64_t stride = (uint64_t)gridDim.x * kThreads, mask = lo_len - 1;
  for (uint64_t t = (uint64_t)blockIdx.x * kThreads + threadIdx.x; t < n; t += stride) {
    fe x[TA];
#pragma unroll
    for (int i = 0; i < TA; i++) x[i] = a.p[i][t];
    fe b = first ? fe_zero() : baggr[t];
#pragma unroll
    for (int j = 0; j < TC; j++) {
      const fe e = fmul(elo[j * lo_len + (t & mask)], ehi[j * hi_len + (t >> h)]);
      b = fadd(b, fmul(sw[j], e));
#pragma unroll
      for (int i = 0; i < TA; i++) acc[i * TC + j] = fadd(acc[i * TC + j], fmul(x[i], e));
    }
    baggr[t] = b;
    if (aw) {
      fe v = fe_zero();
#pragma unroll
      for (int i = 0; i < TA; i++) v = fadd(v, fmul(sw[TC + i], x[i]));
      arr[t] = v;
    }
  }
  __shared__ fe red[TA * TC][kThreads / 32];
  const int wq = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < TA * TC; q++) {
    fe sum = acc[q];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) sum = fadd(sum, shfl_down_fe(sum, d));
    if (lane == 0) red[q][wq] = sum;
  }
  __syncthreads();
  if (threadIdx.x < TA * TC) {
    fe sum = fe_zero();
    for (int k = 0; k < kThreads / 32; k++) sum = fadd(sum, red[threadIdx.x][k]);
    partial[(uint64_t)blockIdx.x * TA * TC + threadIdx.x] = sum;
  }
}

template <int TA, int TC>
void pass_launch(const VecList &a, const fe *elo, const fe *ehi, int h, int lg, uint64_t n, const fe *bw,
                 const fe *aw, int first, fe *arr, fe *baggr, fe *partial, int blocks, cudaStream_t s) {
  aggr_claims_pass_kernel<TA, TC><<<blocks, kThreads, 0, s>>>(a, elo, ehi, h, 1ull << h, 1ull << (lg - h), n, bw,
                                                              aw, first, arr, baggr, partial);
  GBZ_CUDA(cudaGetLastError());
}

}  // namespace

bool aggr_claims_fused(const VecList &a, int k, int c, const fe *elo, const fe *ehi, int h, int lg, uint64_t n,
                       const fe *w, fe *arr, fe *baggr, fe *partial, fe *sums, cudaStream_t s) {
  if (k < 1 || c < 1 || k > 4 || c > 4) return false;
  const int blocks = grid_for(n);
  const uint64_t nlo = 1ull << h, nhi = 1ull << (lg - h);
  fe *tile = partial + (uint64_t)blocks * 16;
  for (int j0 = 0; j0 < c; j0 += 2) {
    const int tc = std::min(2, c - j0);
    const fe *aw = j0 + tc >= c ? w + c : nullptr;  // arr in the last pass
    const fe *el = elo + (uint64_t)j0 * nlo, *eh = ehi + (uint64_t)j0 * nhi;
#define GBZ_AP(A, C) \
    if (k == A && tc == C) pass_launch<A, C>(a, el, eh, h, lg, n, w + j0, aw, j0 == 0, arr, baggr, partial, blocks, s);
    GBZ_AP(1, 1) GBZ_AP(1, 2) GBZ_AP(2, 1) GBZ_AP(2, 2) GBZ_AP(3, 1) GBZ_AP(3, 2) GBZ_AP(4, 1) GBZ_AP(4, 2)
#undef GBZ_AP
    sum_cols_kernel<<<k * tc, kThreads, 0, s>>>(partial, blocks, k * tc, tile);
    GBZ_CUDA(cudaGetLastError());
    // the pass's k x tc sums into columns j0.. of the row-major k x c sums
    GBZ_CUDA(cudaMemcpy2DAsync(sums + j0, sizeof(fe) * c, tile, sizeof(fe) * tc, sizeof(fe) * tc, k,
                               cudaMemcpyDeviceToDevice, s));
  }
  return true;
}

}  // namespace gbz
