// Number-theoretic transform over F_{p^2} for power-of-two lengths.
//
// Replaces fft (utils.cpp:904-964), _fft/__fft (:966-1110) and pfft
// (:1583-1673).  All of them compute out[k] = sum_j in[j] w^{jk} with
// w = getRootOfUnity(logn) (its inverse, plus a 2^-logn scale, for the
// inverse transform); pfft is a 16-thread four-step split of the same
// forward transform.  Exact field arithmetic makes the result independent
// of the factorisation, so the GPU uses its own:
//
//  * lengths up to 2^13: one shared-memory pass;
//  * longer lengths L = N1 * N2 (N1, N2 <= 2^13): the four-step algorithm.
//      pass A: for each column n1 < N1, a length-N2 DFT over x[n1 + N1*n2]
//              (zero beyond n_valid: the Reed-Solomon padding is never
//              read), times omega_L^{n1*k2}, stored at n1 + N1*k2;
//      pass B: for each row k2 < N2, a length-N1 DFT over the row,
//              stored at k2 + N2*k1 (natural order, no bit reversal pass).
//
// Inside a pass every CTA stages B sub-transforms of length S in shared
// memory (bit-reversed on load), runs the radix-2 decimation-in-time
// stages with __syncthreads between them, and applies the outer twiddle
// and the inverse scale on the way out.  Groups of B >= 2 neighbouring
// columns make the strided pass read whole 32-byte sectors.
#include "gbz_internal.cuh"

namespace gbz {

namespace {

constexpr int kSubLog = 13;          // largest sub-transform held in shared memory
constexpr int kTwLoBits = 12;        // outer twiddle table split
constexpr int kThreads = 512;

struct PassArgs {
  const fe *in;
  fe *out;
  uint64_t n_valid;
  uint64_t in_gstride, in_jstride, out_gstride, out_kstride;
  const fe *wsub;    // omega_{2^13}^t, t < 2^12
  const fe *tw_lo;   // omega_L^t, t < 2^12 (nullptr: no outer twiddle)
  const fe *tw_hi;   // omega_L^{2^12 t}
  fe scale;
  int logS, logB, has_scale;
};

__device__ __forceinline__ uint32_t brev_bits(uint32_t x, int bits) {
  return bits ? __brev(x) >> (32 - bits) : 0u;
}

__global__ void __launch_bounds__(kThreads) ntt_pass_kernel(PassArgs a) {
  extern __shared__ fe sm[];
  const int logS = a.logS, logB = a.logB;
  const uint32_t S = 1u << logS, total = S << logB;
  const uint64_t g0 = (uint64_t)blockIdx.x << logB;

  // Load: bit-reversed positions inside each sub-transform.
  if (a.in_jstride == 1) {
    for (uint32_t e = threadIdx.x; e < total; e += kThreads) {
      uint32_t b = e >> logS, j = e & (S - 1);
      uint64_t addr = (g0 + b) * a.in_gstride + j;
      fe v = addr < a.n_valid ? a.in[addr] : fe_zero();
      sm[(b << logS) + brev_bits(j, logS)] = v;
    }
  } else {
    for (uint32_t e = threadIdx.x; e < total; e += kThreads) {
      uint32_t b = e & ((1u << logB) - 1), j = e >> logB;
      uint64_t addr = (g0 + b) * a.in_gstride + (uint64_t)j * a.in_jstride;
      fe v = addr < a.n_valid ? a.in[addr] : fe_zero();
      sm[(b << logS) + brev_bits(j, logS)] = v;
    }
  }
  __syncthreads();

  // Radix-2 DIT stages.
  const uint32_t half_total = total >> 1;
  for (int lh = 0; lh < logS; lh++) {
    const uint32_t h = 1u << lh;
    for (uint32_t t = threadIdx.x; t < half_total; t += kThreads) {
      uint32_t b = t >> (logS - 1), tt = t & ((S >> 1) - 1);
      uint32_t k = tt & (h - 1);
      uint32_t j = (b << logS) + ((tt >> lh) << (lh + 1)) + k;
      fe u = sm[j], v = sm[j + h];
      if (lh) v = fmul(v, a.wsub[k << (kSubLog - 1 - lh)]);
      sm[j] = fadd(u, v);
      sm[j + h] = fsub(u, v);
    }
    __syncthreads();
  }

  // Store with the outer twiddle and scale.
  if (a.out_kstride == 1) {
    for (uint32_t e = threadIdx.x; e < total; e += kThreads) {
      uint32_t b = e >> logS, k = e & (S - 1);
      fe v = sm[e];
      if (a.tw_lo) {
        uint64_t ex = (g0 + b) * k;
        v = fmul(v, fmul(a.tw_lo[ex & ((1u << kTwLoBits) - 1)], a.tw_hi[ex >> kTwLoBits]));
      }
      if (a.has_scale) v = fmul(v, a.scale);
      a.out[(g0 + b) * a.out_gstride + k] = v;
    }
  } else {
    for (uint32_t e = threadIdx.x; e < total; e += kThreads) {
      uint32_t b = e & ((1u << logB) - 1), k = e >> logB;
      fe v = sm[(b << logS) + k];
      if (a.tw_lo) {
        uint64_t ex = (g0 + b) * k;
        v = fmul(v, fmul(a.tw_lo[ex & ((1u << kTwLoBits) - 1)], a.tw_hi[ex >> kTwLoBits]));
      }
      if (a.has_scale) v = fmul(v, a.scale);
      a.out[(g0 + b) * a.out_gstride + (uint64_t)k * a.out_kstride] = v;
    }
  }
}

// omega_{2^13}^t for t < 2^12, per direction; shared by every length.
fe *g_wsub[2] = {nullptr, nullptr};
int g_wsub_device = -1;

void ensure_wsub() {
  int dev;
  GBZ_CUDA(cudaGetDevice(&dev));
  if (g_wsub[0] && g_wsub_device == dev) return;
  const int n = 1 << (kSubLog - 1);
  std::vector<fe> h(n);
  for (int dir = 0; dir < 2; dir++) {
    fe w = root_of_unity(kSubLog);
    if (dir) w = finv(w);
    fe x = fe_one();
    for (int t = 0; t < n; t++) { h[t] = x; x = fmul(x, w); }
    GBZ_CUDA(cudaMalloc(&g_wsub[dir], sizeof(fe) * n));
    GBZ_CUDA(cudaMemcpy(g_wsub[dir], h.data(), sizeof(fe) * n, cudaMemcpyHostToDevice));
  }
  g_wsub_device = dev;
  GBZ_CUDA(cudaFuncSetAttribute(ntt_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (1 << kSubLog) * (int)sizeof(fe)));
}

void launch_pass(const PassArgs &a, uint64_t groups, cudaStream_t s) {
  uint64_t blocks = groups >> a.logB;
  size_t smem = sizeof(fe) << (a.logS + a.logB);
  ntt_pass_kernel<<<(unsigned)blocks, kThreads, smem, s>>>(a);
  GBZ_CUDA(cudaGetLastError());
}

}  // namespace

void ntt_tables_build(NttTables &t, int logn) {
  ensure_wsub();
  t.logn = logn;
  t.sub_fwd = g_wsub[0];
  t.sub_inv = g_wsub[1];
  t.inv_len = finv(fe_make(1ull << logn, 0));
  if (logn <= kSubLog) return;
  const uint64_t L = 1ull << logn;
  const int nlo = 1 << kTwLoBits;
  const uint64_t nhi = (L >> kTwLoBits) > 0 ? (L >> kTwLoBits) : 1;
  std::vector<fe> lo(nlo), hi(nhi);
  for (int dir = 0; dir < 2; dir++) {
    fe w = root_of_unity(logn);
    if (dir) w = finv(w);
    fe x = fe_one();
    for (int i = 0; i < nlo; i++) { lo[i] = x; x = fmul(x, w); }
    fe w12 = x;  // w^(2^12)
    x = fe_one();
    for (uint64_t i = 0; i < nhi; i++) { hi[i] = x; x = fmul(x, w12); }
    fe **plo = dir ? &t.lo_inv : &t.lo_fwd, **phi = dir ? &t.hi_inv : &t.hi_fwd;
    GBZ_CUDA(cudaMalloc(plo, sizeof(fe) * nlo));
    GBZ_CUDA(cudaMalloc(phi, sizeof(fe) * nhi));
    GBZ_CUDA(cudaMemcpy(*plo, lo.data(), sizeof(fe) * nlo, cudaMemcpyHostToDevice));
    GBZ_CUDA(cudaMemcpy(*phi, hi.data(), sizeof(fe) * nhi, cudaMemcpyHostToDevice));
  }
}

int ntt_launch_count(int logn) { return logn <= kSubLog ? 1 : 2; }

void ntt_tables_free(NttTables &t) {
  cudaFree(t.lo_fwd);
  cudaFree(t.hi_fwd);
  cudaFree(t.lo_inv);
  cudaFree(t.hi_inv);
  t.lo_fwd = t.hi_fwd = t.lo_inv = t.hi_inv = nullptr;
  t.logn = -1;
}

void ntt_launch(const NttTables &t, const fe *in, uint64_t n_valid, fe *out, fe *tmp, bool inverse,
                cudaStream_t s) {
  const int logn = t.logn;
  const uint64_t L = 1ull << logn;
  if (n_valid > L) n_valid = L;
  PassArgs a{};
  a.wsub = inverse ? t.sub_inv : t.sub_fwd;
  a.scale = t.inv_len;
  if (logn <= kSubLog) {
    a.in = in;
    a.out = out;
    a.n_valid = n_valid;
    a.in_gstride = L;
    a.in_jstride = 1;
    a.out_gstride = L;
    a.out_kstride = 1;
    a.logS = logn;
    a.logB = 0;
    a.has_scale = inverse;
    a.tw_lo = nullptr;
    a.tw_hi = nullptr;
    launch_pass(a, 1, s);
    return;
  }
  const int k1 = (logn + 1) / 2;  // pass B (contiguous rows)
  const int k2 = logn - k1;       // pass A (strided columns)
  const uint64_t N1 = 1ull << k1, N2 = 1ull << k2;
  // pass A: columns n1 < N1, length N2, stride N1
  a.in = in;
  a.out = tmp;
  a.n_valid = n_valid;
  a.in_gstride = 1;
  a.in_jstride = N1;
  a.out_gstride = 1;
  a.out_kstride = N1;
  a.logS = k2;
  a.logB = k2 <= 12 ? (k2 >= 12 ? 1 : 12 - k2) : 0;
  if ((1ull << a.logB) > N1) a.logB = k1;
  a.tw_lo = inverse ? t.lo_inv : t.lo_fwd;
  a.tw_hi = inverse ? t.hi_inv : t.hi_fwd;
  a.has_scale = 0;
  launch_pass(a, N1, s);
  // pass B: rows k2 < N2, length N1, contiguous
  PassArgs b = a;
  b.in = tmp;
  b.out = out;
  b.n_valid = L;
  b.in_gstride = N1;
  b.in_jstride = 1;
  b.out_gstride = 1;
  b.out_kstride = N2;
  b.logS = k1;
  b.logB = k1 >= 12 ? (k1 == 12 ? 1 : 0) : 12 - k1;
  if ((1ull << b.logB) > N2) b.logB = k2;
  b.tw_lo = nullptr;
  b.tw_hi = nullptr;
  b.has_scale = inverse;
  launch_pass(b, N2, s);
}

}  // namespace gbz
