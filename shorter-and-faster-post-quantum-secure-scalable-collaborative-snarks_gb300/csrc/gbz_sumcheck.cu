// Sumcheck round kernels, the eq (beta) table and the WHIR beta update.
//
// Round message (coSumcheck_MPI.cpp:199, Whir.cpp:215-221,
// delegate_protocol.cpp:16-21): over pairs j of two vectors,
//   H(x) = sum_j (a1 x + b1)(a2 x + b2),  a = v[2j+1] - v[2j], b = v[2j],
// so H = (sum a1 a2, sum a1 b2 + b1 a2, sum b1 b2).  With
// D = v1[2j+1] v2[2j+1] the middle term is D - A - C, three products per
// pair instead of four (exact arithmetic, same value).
// Fold (coSumcheck_MPI.cpp:215-218, Whir.cpp:223-231):
//   v[j] = r (v[2j+1] - v[2j]) + v[2j].
// The fold of round i and the message of round i+1 are one pass: each
// thread reads four consecutive entries of both vectors, writes the two
// folded entries of each and accumulates the next message from them.
#include <algorithm>

#include "gbz_internal.cuh"

namespace gbz {

namespace {

constexpr int kScThreads = 256;

__device__ __forceinline__ fe shfl_down_fe(fe v, int d) {
  fe r;
  r.re = __shfl_down_sync(0xffffffffu, v.re, d);
  r.im = __shfl_down_sync(0xffffffffu, v.im, d);
  return r;
}

// Block-wide sum of three field elements; result valid in thread 0.
__device__ void block_sum3(fe &x, fe &y, fe &z) {
  __shared__ fe red[3][kScThreads / 32];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    x = fadd(x, shfl_down_fe(x, d));
    y = fadd(y, shfl_down_fe(y, d));
    z = fadd(z, shfl_down_fe(z, d));
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { red[0][w] = x; red[1][w] = y; red[2][w] = z; }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    x = lane < nw ? red[0][lane] : fe_zero();
    y = lane < nw ? red[1][lane] : fe_zero();
    z = lane < nw ? red[2][lane] : fe_zero();
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      x = fadd(x, shfl_down_fe(x, d));
      y = fadd(y, shfl_down_fe(y, d));
      z = fadd(z, shfl_down_fe(z, d));
    }
  }
}

__device__ __forceinline__ void acc_pair(fe a0, fe a1, fe b0, fe b1, fe &A, fe &C, fe &D) {
  A = fadd(A, fmul(fsub(a1, a0), fsub(b1, b0)));
  C = fadd(C, fmul(a0, b0));
  D = fadd(D, fmul(a1, b1));
}

// partial[3*blk + {0,1,2}] = (sum A, sum C, sum D) of the block.
__global__ void __launch_bounds__(kScThreads)
sc_reduce_kernel(const fe *__restrict__ a, const fe *__restrict__ b, uint64_t pairs, fe *partial) {
  fe A = fe_zero(), C = fe_zero(), D = fe_zero();
  const uint64_t stride = (uint64_t)gridDim.x * kScThreads;
  for (uint64_t j = (uint64_t)blockIdx.x * kScThreads + threadIdx.x; j < pairs; j += stride) {
    fe a0 = a[2 * j], a1 = a[2 * j + 1], b0 = b[2 * j], b1 = b[2 * j + 1];
    acc_pair(a0, a1, b0, b1, A, C, D);
  }
  block_sum3(A, C, D);
  if (threadIdx.x == 0) {
    partial[3 * blockIdx.x] = A;
    partial[3 * blockIdx.x + 1] = C;
    partial[3 * blockIdx.x + 2] = D;
  }
}

// Fold (a, b) of length m by *chal into (a2, b2) of length m/2; when
// reduce, accumulate the message of the folded pair sequence.
__global__ void __launch_bounds__(kScThreads)
sc_fold_kernel(const fe *__restrict__ a, const fe *__restrict__ b, uint64_t m, const fe *chal,
               fe *__restrict__ a2, fe *__restrict__ b2, int reduce, fe *partial) {
  const fe r = *chal;
  fe A = fe_zero(), C = fe_zero(), D = fe_zero();
  const uint64_t stride = (uint64_t)gridDim.x * kScThreads;
  const uint64_t quads = m / 4;
  for (uint64_t t = (uint64_t)blockIdx.x * kScThreads + threadIdx.x; t < quads; t += stride) {
    fe x0 = a[4 * t], x1 = a[4 * t + 1], x2 = a[4 * t + 2], x3 = a[4 * t + 3];
    fe y0 = b[4 * t], y1 = b[4 * t + 1], y2 = b[4 * t + 2], y3 = b[4 * t + 3];
    fe fa0 = fadd(fmul(r, fsub(x1, x0)), x0), fa1 = fadd(fmul(r, fsub(x3, x2)), x2);
    fe fb0 = fadd(fmul(r, fsub(y1, y0)), y0), fb1 = fadd(fmul(r, fsub(y3, y2)), y2);
    a2[2 * t] = fa0; a2[2 * t + 1] = fa1;
    b2[2 * t] = fb0; b2[2 * t + 1] = fb1;
    if (reduce) acc_pair(fa0, fa1, fb0, fb1, A, C, D);
  }
  if (m == 2 && blockIdx.x == 0 && threadIdx.x == 0) {  // fold to a single entry
    a2[0] = fadd(fmul(r, fsub(a[1], a[0])), a[0]);
    b2[0] = fadd(fmul(r, fsub(b[1], b[0])), b[0]);
  }
  if (!reduce) return;
  block_sum3(A, C, D);
  if (threadIdx.x == 0) {
    partial[3 * blockIdx.x] = A;
    partial[3 * blockIdx.x + 1] = C;
    partial[3 * blockIdx.x + 2] = D;
  }
}

// Two WHIR sumcheck rounds in one pass (Whir.cpp:215-231 twice): the
// challenges r0, r1 are drawn before the round messages exist (F::_random),
// so a thread takes four consecutive entries of both vectors, adds the two
// pairs to the first round's message, folds them by r0, adds the folded pair
// to the second round's message and folds it by r1 into (a4, b4) of length
// m/4.  One read of (a, b) instead of three passes.
__global__ void __launch_bounds__(kScThreads)
sc_fold2_kernel(const fe *__restrict__ a, const fe *__restrict__ b, uint64_t m, const fe *chal0, const fe *chal1,
                fe *__restrict__ a4, fe *__restrict__ b4, fe *partial0, fe *partial1, BStr bs) {
  const uint32_t pb = blockIdx.y;
  a = badv(a, bs.s[0], pb);
  b = badv(b, bs.s[1], pb);
  chal0 = badv(chal0, bs.s[2], pb);
  chal1 = badv(chal1, bs.s[3], pb);
  a4 = badv(a4, bs.s[4], pb);
  b4 = badv(b4, bs.s[5], pb);
  partial0 = badv(partial0, bs.s[6], pb);
  partial1 = badv(partial1, bs.s[7], pb);
  const fe r0 = *chal0, r1 = *chal1;
  fe A0 = fe_zero(), C0 = fe_zero(), D0 = fe_zero(), A1 = fe_zero(), C1 = fe_zero(), D1 = fe_zero();
  const uint64_t stride = (uint64_t)gridDim.x * kScThreads;
  const uint64_t quads = m / 4;
  for (uint64_t t = (uint64_t)blockIdx.x * kScThreads + threadIdx.x; t < quads; t += stride) {
    const fe x0 = a[4 * t], x1 = a[4 * t + 1], x2 = a[4 * t + 2], x3 = a[4 * t + 3];
    const fe y0 = b[4 * t], y1 = b[4 * t + 1], y2 = b[4 * t + 2], y3 = b[4 * t + 3];
    acc_pair(x0, x1, y0, y1, A0, C0, D0);
    acc_pair(x2, x3, y2, y3, A0, C0, D0);
    const fe fa0 = fadd(fmul(r0, fsub(x1, x0)), x0), fa1 = fadd(fmul(r0, fsub(x3, x2)), x2);
    const fe fb0 = fadd(fmul(r0, fsub(y1, y0)), y0), fb1 = fadd(fmul(r0, fsub(y3, y2)), y2);
    acc_pair(fa0, fa1, fb0, fb1, A1, C1, D1);
    a4[t] = fadd(fmul(r1, fsub(fa1, fa0)), fa0);
    b4[t] = fadd(fmul(r1, fsub(fb1, fb0)), fb0);
  }
  block_sum3(A0, C0, D0);
  if (threadIdx.x == 0) {
    partial0[3 * blockIdx.x] = A0;
    partial0[3 * blockIdx.x + 1] = C0;
    partial0[3 * blockIdx.x + 2] = D0;
  }
  __syncthreads();  // block_sum3's shared scratch is reused
  block_sum3(A1, C1, D1);
  if (threadIdx.x == 0) {
    partial1[3 * blockIdx.x] = A1;
    partial1[3 * blockIdx.x + 1] = C1;
    partial1[3 * blockIdx.x + 2] = D1;
  }
}

// The same two rounds for the first WHIR iteration, whose b is the eq
// vector of the sumcheck challenges c (precompute_beta, utils.cpp:198-243):
// b[4t + 2 x1 + x0] = eq1(c0, x0) eq1(c1, x1) E2[t] with E2 the eq table of
// c2.. (m/4 entries), so b is never read.  Per pair the messages need only
// S0 = sum a0 g and S1 = sum a1 g (g the pair's factor without eq1(c0, .)):
// A = (e1 - e0)(S1 - S0), C = e0 S0, D = e1 S1 (e_x = eq1(c0, x)), and after
// the fold by r0 the pair's b is lambda0 eq1(c1, x1) E2[t], lambda0 =
// eq1(c0, r0); b4 = lambda0 lambda1 E2 (lambda1 = eq1(c1, r1)).
__global__ void __launch_bounds__(kScThreads)
sc_fold2_eq_kernel(const fe *__restrict__ a, const fe *__restrict__ E2, uint64_t m, const fe *c, const fe *chal0,
                   const fe *chal1, fe *__restrict__ a4, fe *__restrict__ b4, fe *partial0, fe *partial1, BStr bs) {
  const uint32_t pb = blockIdx.y;
  a = badv(a, bs.s[0], pb);
  E2 = badv(E2, bs.s[1], pb);
  c = badv(c, bs.s[2], pb);
  chal0 = badv(chal0, bs.s[3], pb);
  chal1 = badv(chal1, bs.s[4], pb);
  a4 = badv(a4, bs.s[5], pb);
  b4 = badv(b4, bs.s[6], pb);
  partial0 = badv(partial0, bs.s[7], pb);
  partial1 = badv(partial1, bs.s[8], pb);
  const fe r0 = *chal0, r1 = *chal1, c0 = c[0], c1 = c[1];
  const fe e0 = fsub(fe_one(), c0), f0 = fsub(fe_one(), c1);
  const fe lam0 = fadd(fmul(r0, fsub(c0, e0)), e0), lam1 = fadd(fmul(r1, fsub(c1, f0)), f0);
  const fe lam = fmul(lam0, lam1);
  fe S0 = fe_zero(), S1 = fe_zero(), T0 = fe_zero(), T1 = fe_zero();
  const uint64_t stride = (uint64_t)gridDim.x * kScThreads;
  const uint64_t quads = m / 4;
  for (uint64_t t = (uint64_t)blockIdx.x * kScThreads + threadIdx.x; t < quads; t += stride) {
    const fe x0 = a[4 * t], x1 = a[4 * t + 1], x2 = a[4 * t + 2], x3 = a[4 * t + 3];
    const fe E = E2[t];
    const fe g0 = fmul(f0, E), g1 = fmul(c1, E);
    fe fa0, fa1;
    if (!(x0.im | x1.im | x2.im | x3.im)) {
      // base-field entries (the witness of the configurations): products
      // with a base-field factor need two of the four partial products
      S0 = fadd(S0, fadd(fmul_base(g0, x0.re), fmul_base(g1, x2.re)));
      S1 = fadd(S1, fadd(fmul_base(g0, x1.re), fmul_base(g1, x3.re)));
      fa0 = fadd(fmul_base(r0, subp(x1.re, x0.re)), x0);
      fa1 = fadd(fmul_base(r0, subp(x3.re, x2.re)), x2);
    } else {
      S0 = fadd(S0, fadd(fmul(x0, g0), fmul(x2, g1)));
      S1 = fadd(S1, fadd(fmul(x1, g0), fmul(x3, g1)));
      fa0 = fadd(fmul(r0, fsub(x1, x0)), x0);
      fa1 = fadd(fmul(r0, fsub(x3, x2)), x2);
    }
    T0 = fadd(T0, fmul(fa0, E));
    T1 = fadd(T1, fmul(fa1, E));
    a4[t] = fadd(fmul(r1, fsub(fa1, fa0)), fa0);
    b4[t] = fmul(lam, E);
  }
  fe Z = fe_zero();
  block_sum3(S0, S1, Z);
  if (threadIdx.x == 0) {
    partial0[3 * blockIdx.x] = fmul(fsub(c0, e0), fsub(S1, S0));
    partial0[3 * blockIdx.x + 1] = fmul(e0, S0);
    partial0[3 * blockIdx.x + 2] = fmul(c0, S1);
  }
  __syncthreads();  // block_sum3's shared scratch is reused
  Z = fe_zero();
  block_sum3(T0, T1, Z);
  if (threadIdx.x == 0) {
    partial1[3 * blockIdx.x] = fmul(lam0, fmul(fsub(c1, f0), fsub(T1, T0)));
    partial1[3 * blockIdx.x + 1] = fmul(lam0, fmul(f0, T0));
    partial1[3 * blockIdx.x + 2] = fmul(lam0, fmul(c1, T1));
  }
}

// Sumcheck of sum_x w(x) eq(z, x) without folding the eq vector.  After i
// rounds the folded eq vector is epre * eq1(z_i, x_0) * E_i[x'], E_i the eq
// table of z_{i+1..} (eq1(z, x) = z x + (1 - z)(1 - x)), so the round
// polynomial is epre * eq1(z_i, X) * S(X) with S(X) = sum_j l_j(X) E_i[j]:
// only S(0) = sum w[2j] E_i[j] and S(1) = sum w[2j+1] E_i[j] are summed
// over the vector (the same polynomial as the pairwise products of the
// reference's loop, computed with half the reads and multiplies).
// E_{i+1}[t] = E_i[2t] + E_i[2t+1].
// partial[3 blk + {0, 1, 2}] = (S0, S1, 0).
__global__ void __launch_bounds__(kScThreads)
sc_eq_reduce_kernel(const fe *__restrict__ a, const fe *__restrict__ E, uint64_t pairs, fe *partial, BStr bs) {
  const uint32_t pb = blockIdx.y;
  a = badv(a, bs.s[0], pb);
  E = badv(E, bs.s[1], pb);
  partial = badv(partial, bs.s[2], pb);
  fe S0 = fe_zero(), S1 = fe_zero(), Z = fe_zero();
  const uint64_t stride = (uint64_t)gridDim.x * kScThreads;
  for (uint64_t j = (uint64_t)blockIdx.x * kScThreads + threadIdx.x; j < pairs; j += stride) {
    const fe e = E[j], w0 = a[2 * j], w1 = a[2 * j + 1];
    if (!(w0.im | w1.im)) {  // base-field entries: two partial products each
      S0 = fadd(S0, fmul_base(e, w0.re));
      S1 = fadd(S1, fmul_base(e, w1.re));
    } else {
      S0 = fadd(S0, fmul(w0, e));
      S1 = fadd(S1, fmul(w1, e));
    }
  }
  block_sum3(S0, S1, Z);
  if (threadIdx.x == 0) {
    partial[3 * blockIdx.x] = S0;
    partial[3 * blockIdx.x + 1] = S1;
    partial[3 * blockIdx.x + 2] = fe_zero();
  }
}

// Fold a (length m) by *chal into a2, E (length m/2) into E2 (length m/4)
// by pairwise sums, and (reduce) the S sums of the folded pairs with E2.
__global__ void __launch_bounds__(kScThreads)
sc_eq_fold_kernel(const fe *__restrict__ a, uint64_t m, const fe *chal, fe *__restrict__ a2,
                  const fe *__restrict__ E, fe *__restrict__ E2, int reduce, fe *partial, BStr bs) {
  const uint32_t pb = blockIdx.y;
  a = badv(a, bs.s[0], pb);
  chal = badv(chal, bs.s[1], pb);
  a2 = badv(a2, bs.s[2], pb);
  E = badv(E, bs.s[3], pb);
  E2 = badv(E2, bs.s[4], pb);
  partial = badv(partial, bs.s[5], pb);
  const fe r = *chal;
  fe S0 = fe_zero(), S1 = fe_zero(), Z = fe_zero();
  const uint64_t stride = (uint64_t)gridDim.x * kScThreads;
  const uint64_t quads = m / 4;
  for (uint64_t t = (uint64_t)blockIdx.x * kScThreads + threadIdx.x; t < quads; t += stride) {
    const fe x0 = a[4 * t], x1 = a[4 * t + 1], x2 = a[4 * t + 2], x3 = a[4 * t + 3];
    const fe e0 = E[2 * t], e1 = E[2 * t + 1];
    fe f0, f1;
    if (!(x0.im | x1.im | x2.im | x3.im)) {  // base-field entries (the first fold of the witness)
      f0 = fadd(fmul_base(r, subp(x1.re, x0.re)), x0);
      f1 = fadd(fmul_base(r, subp(x3.re, x2.re)), x2);
    } else {
      f0 = fadd(fmul(r, fsub(x1, x0)), x0);
      f1 = fadd(fmul(r, fsub(x3, x2)), x2);
    }
    a2[2 * t] = f0;
    a2[2 * t + 1] = f1;
    const fe e = fadd(e0, e1);
    if (reduce) {
      E2[t] = e;
      S0 = fadd(S0, fmul(f0, e));
      S1 = fadd(S1, fmul(f1, e));
    }
  }
  if (m == 2 && blockIdx.x == 0 && threadIdx.x == 0) a2[0] = fadd(fmul(r, fsub(a[1], a[0])), a[0]);
  if (!reduce) return;
  block_sum3(S0, S1, Z);
  if (threadIdx.x == 0) {
    partial[3 * blockIdx.x] = S0;
    partial[3 * blockIdx.x + 1] = S1;
    partial[3 * blockIdx.x + 2] = fe_zero();
  }
}

// out = (a, b, c) of the round message from (A, C, D) partials.
__global__ void __launch_bounds__(kScThreads) sc_sum_kernel(const fe *partial, int blocks, fe *out) {
  fe A = fe_zero(), C = fe_zero(), D = fe_zero();
  for (int i = threadIdx.x; i < blocks; i += kScThreads) {
    A = fadd(A, partial[3 * i]);
    C = fadd(C, partial[3 * i + 1]);
    D = fadd(D, partial[3 * i + 2]);
  }
  block_sum3(A, C, D);
  if (threadIdx.x == 0) {
    out[0] = A;
    out[1] = fsub(fsub(D, A), C);
    out[2] = C;
  }
}

// precompute_beta, one CTA per block of 2^11 consecutive entries: thread 0
// forms the product over the index bits from 11 up, then the CTA doubles the
// table in shared memory from bit 10 down to bit 0 (T[2j+1] = T[j] r_i,
// T[2j] = T[j] - T[j] r_i, one product per entry) and writes the block with
// coalesced 16-byte stores.
constexpr int kBetaBlockLog = 11;
__global__ void __launch_bounds__(256) beta_block_kernel(const fe *r, int nr, fe *B, BStr bs) {
  __shared__ fe T[1 << kBetaBlockLog];
  __shared__ fe rs[64];
  r = badv(r, bs.s[0], blockIdx.y);
  B = badv(B, bs.s[1], blockIdx.y);
  const int low = nr < kBetaBlockLog ? nr : kBetaBlockLog;
  if ((int)threadIdx.x < nr) rs[threadIdx.x] = r[threadIdx.x];
  __syncthreads();
  if (threadIdx.x == 0) {
    fe pre = fe_one();
    const uint64_t hi = (uint64_t)blockIdx.x;
    for (int i = low; i < nr; i++) pre = fmul(pre, ((hi >> (i - low)) & 1) ? rs[i] : fsub(fe_one(), rs[i]));
    T[0] = pre;
  }
  __syncthreads();
  for (int i = low - 1; i >= 0; i--) {
    const int len = 1 << (low - 1 - i);  // entries before this level (at most 2^10)
    const fe ri = rs[i];
    fe v[4];
    int cnt = 0;
    for (int j = threadIdx.x; j < len; j += blockDim.x) v[cnt++] = T[j];
    __syncthreads();
    cnt = 0;
    for (int j = threadIdx.x; j < len; j += blockDim.x) {
      const fe t = v[cnt++];
      const fe x = fmul(t, ri);
      T[2 * j + 1] = x;
      T[2 * j] = fsub(t, x);
    }
    __syncthreads();
  }
  fe *o = B + ((uint64_t)blockIdx.x << low);
  for (int j = threadIdx.x; j < (1 << low); j += blockDim.x) o[j] = T[j];
}

// Tables of 2^15 entries or more: a CTA writes 16 blocks of 2^11 entries.
// The table is the tensor product of the eq table LO over the 11 low
// variables (built once per CTA by doubling in shared memory) and the
// products over the high variables of each block (16 threads, one block
// each), so every output entry costs one product and the serial part of a
// CTA is amortised over 2^15 entries.
constexpr int kBetaChunksLog = 4;  // at most 16 blocks of 2^11 entries per CTA
__global__ void __launch_bounds__(256) beta_tensor_kernel(const fe *r, int nr, int chunks_log, fe *B, BStr bs) {
  __shared__ fe T[1 << kBetaBlockLog];
  __shared__ fe hi_pre[1 << kBetaChunksLog];
  __shared__ fe rs[64];
  r = badv(r, bs.s[0], blockIdx.y);
  B = badv(B, bs.s[1], blockIdx.y);
  if ((int)threadIdx.x < nr) rs[threadIdx.x] = r[threadIdx.x];
  __syncthreads();
  if (threadIdx.x < (1u << chunks_log)) {
    const uint64_t c = ((uint64_t)blockIdx.x << chunks_log) + threadIdx.x;  // block of 2^11 entries
    fe pre = fe_one();
    for (int i = kBetaBlockLog; i < nr; i++)
      pre = fmul(pre, ((c >> (i - kBetaBlockLog)) & 1) ? rs[i] : fsub(fe_one(), rs[i]));
    hi_pre[threadIdx.x] = pre;
  }
  if (threadIdx.x == 32) T[0] = fe_one();
  __syncthreads();
  for (int i = kBetaBlockLog - 1; i >= 0; i--) {
    const int len = 1 << (kBetaBlockLog - 1 - i);
    const fe ri = rs[i];
    fe v[4];
    int cnt = 0;
    for (int j = threadIdx.x; j < len; j += blockDim.x) v[cnt++] = T[j];
    __syncthreads();
    cnt = 0;
    for (int j = threadIdx.x; j < len; j += blockDim.x) {
      const fe t = v[cnt++];
      const fe x = fmul(t, ri);
      T[2 * j + 1] = x;
      T[2 * j] = fsub(t, x);
    }
    __syncthreads();
  }
  fe lo[(1 << kBetaBlockLog) / 256];
#pragma unroll
  for (int k = 0; k < (1 << kBetaBlockLog) / 256; k++) lo[k] = T[threadIdx.x + 256 * k];
  fe *o = B + ((uint64_t)blockIdx.x << (kBetaBlockLog + chunks_log));
  for (int c = 0; c < (1 << chunks_log); c++) {
    const fe h = hi_pre[c];
#pragma unroll
    for (int k = 0; k < (1 << kBetaBlockLog) / 256; k++)
      o[((uint64_t)c << kBetaBlockLog) + threadIdx.x + 256 * k] = fmul(h, lo[k]);
  }
}

// update_betas: b[j] += sum_i c_i * w_i^j.  A CTA owns kUbSpan = 256
// consecutive entries: lane L of every warp owns the kUbPer = 8 entries
// starting at cta0 + 8L, and warp g takes the queries i = g (mod 8), so the
// l * 256 multiply-adds of a CTA are spread over all its threads; the eight
// warps' partial sums are added in shared memory.  A thread starts each of
// its queries' geometric runs from s_i * pw_i[L] (s_i = c_i w_i^{cta0},
// pw_i[L] = w_i^{8L}) and steps it by w_i.
constexpr int kUbThreads = 256;
constexpr int kUbWarps = kUbThreads / 32;
constexpr int kUbPer = 8;
constexpr int kUbSpan = 32 * kUbPer;

__global__ void __launch_bounds__(kUbThreads) ub_table_kernel(const ProofState *st, int l, fe *pw, BStr bs) {
  // pw[i*32 + L] = w_i^(L * kUbPer)
  st = badv(st, bs.s[0], blockIdx.y);
  pw = badv(pw, bs.s[1], blockIdx.y);
  const int i = blockIdx.x, t = threadIdx.x;
  if (i >= l || t >= 32) return;
  pw[i * 32 + t] = fpow(st->omega_q[i], (uint64_t)t * kUbPer);
}

__global__ void __launch_bounds__(kUbThreads)
ub_kernel(fe *b, uint64_t nb, const ProofState *st, int l, const fe *pw, BStr bs) {
  __shared__ fe s_start[kMaxQueries], s_w[kMaxQueries];
  b = badv(b, bs.s[0], blockIdx.y);
  st = badv(st, bs.s[1], blockIdx.y);
  pw = badv(pw, bs.s[2], blockIdx.y);
  __shared__ fe part[kUbWarps][kUbSpan];
  const uint64_t cta0 = (uint64_t)blockIdx.x * kUbSpan;
  for (int i = threadIdx.x; i < l; i += kUbThreads) {
    const fe w = st->omega_q[i];
    s_w[i] = w;
    s_start[i] = fmul(st->comb[i], fpow(w, cta0));
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  fe acc[kUbPer];
#pragma unroll
  for (int k = 0; k < kUbPer; k++) acc[k] = fe_zero();
  for (int i = warp; i < l; i += kUbWarps) {
    const fe w = s_w[i];
    fe d = fmul(s_start[i], pw[i * 32 + lane]);
#pragma unroll
    for (int k = 0; k < kUbPer; k++) {
      acc[k] = fadd(acc[k], d);
      d = fmul(d, w);
    }
  }
#pragma unroll
  for (int k = 0; k < kUbPer; k++) part[warp][lane * kUbPer + k] = acc[k];
  __syncthreads();
  // thread t finishes entry cta0 + t
  const uint64_t j = cta0 + threadIdx.x;
  if (j >= nb) return;
  fe sum = part[0][threadIdx.x];
#pragma unroll
  for (int g = 1; g < kUbWarps; g++) sum = fadd(sum, part[g][threadIdx.x]);
  b[j] = fadd(b[j], sum);
}

}  // namespace

int sc_blocks(uint64_t pairs) {
  uint64_t want = (pairs + kScThreads - 1) / kScThreads;
  const uint64_t cap = 152 * 8;  // 8 CTAs per SM on 152 SMs, grid-stride beyond that
  if (want > cap) want = cap;
  return want ? (int)want : 1;
}

void sc_step_launch(const fe *a, const fe *b, uint64_t m, const fe *chal, fe *a2, fe *b2, bool reduce,
                    fe *partial, int blocks, cudaStream_t s) {
  if (!chal) {
    sc_reduce_kernel<<<blocks, kScThreads, 0, s>>>(a, b, m / 2, partial);
  } else {
    sc_fold_kernel<<<blocks, kScThreads, 0, s>>>(a, b, m, chal, a2, b2, reduce ? 1 : 0, partial);
  }
  GBZ_CUDA(cudaGetLastError());
}

void sc_fold2_launch(const fe *a, const fe *b, uint64_t m, const fe *chal0, const fe *chal1, fe *a4, fe *b4,
                     fe *partial0, fe *partial1, int blocks, cudaStream_t s, int batch, const BStr &bs) {
  if (m < 4) throw ArgError("two-round fold needs at least 4 entries");
  sc_fold2_kernel<<<dim3(blocks, batch), kScThreads, 0, s>>>(a, b, m, chal0, chal1, a4, b4, partial0, partial1, bs);
  GBZ_CUDA(cudaGetLastError());
}

void sc_fold2_eq_launch(const fe *a, const fe *E2, uint64_t m, const fe *c, const fe *chal0, const fe *chal1, fe *a4,
                        fe *b4, fe *partial0, fe *partial1, int blocks, cudaStream_t s, int batch, const BStr &bs) {
  if (m < 4) throw ArgError("two-round fold needs at least 4 entries");
  sc_fold2_eq_kernel<<<dim3(blocks, batch), kScThreads, 0, s>>>(a, E2, m, c, chal0, chal1, a4, b4, partial0,
                                                                partial1, bs);
  GBZ_CUDA(cudaGetLastError());
}

void sc_eq_step_launch(const fe *a, const fe *E, uint64_t m, const fe *chal, fe *a2, fe *E2, bool reduce,
                       fe *partial, int blocks, cudaStream_t s, int batch, const BStr &bs) {
  // bs: strides of (a, E, chal, a2, E2, partial)
  if (!chal) {
    BStr r;
    r.s[0] = bs.s[0];
    r.s[1] = bs.s[1];
    r.s[2] = bs.s[5];
    sc_eq_reduce_kernel<<<dim3(blocks, batch), kScThreads, 0, s>>>(a, E, m / 2, partial, r);
  } else {
    BStr f;
    f.s[0] = bs.s[0];
    f.s[1] = bs.s[2];
    f.s[2] = bs.s[3];
    f.s[3] = bs.s[1];
    f.s[4] = bs.s[4];
    f.s[5] = bs.s[5];
    sc_eq_fold_kernel<<<dim3(blocks, batch), kScThreads, 0, s>>>(a, m, chal, a2, E, E2, reduce ? 1 : 0, partial, f);
  }
  GBZ_CUDA(cudaGetLastError());
}

void sc_sum_launch(const fe *partial, int blocks, fe *out3, cudaStream_t s) {
  sc_sum_kernel<<<1, kScThreads, 0, s>>>(partial, blocks, out3);
  GBZ_CUDA(cudaGetLastError());
}

void beta_launch(const fe *r, int nr, fe *B, cudaStream_t s, int batch, uint64_t r_stride, uint64_t B_stride) {
  if (nr < 0 || nr > 60) throw ArgError("beta table: bad number of variables");
  BStr bs;
  bs.s[0] = r_stride;
  bs.s[1] = B_stride;
  if (nr >= kBetaBlockLog + 4) {
    // enough CTAs to cover the SMs (at least 2^9), up to 16 blocks each
    const int chunks_log = std::max(0, std::min(kBetaChunksLog, nr - kBetaBlockLog - 9));
    beta_tensor_kernel<<<dim3((unsigned)(1ull << (nr - kBetaBlockLog - chunks_log)), batch), 256, 0, s>>>(
        r, nr, chunks_log, B, bs);
    GBZ_CUDA(cudaGetLastError());
    return;
  }
  const int low = nr < kBetaBlockLog ? nr : kBetaBlockLog;
  beta_block_kernel<<<dim3((unsigned)(1ull << (nr - low)), batch), 256, 0, s>>>(r, nr, B, bs);
  GBZ_CUDA(cudaGetLastError());
}

void update_betas_launch(fe *b, uint64_t nb, const ProofState *st, int l, fe *pw_scratch, cudaStream_t s, int batch,
                         uint64_t b_stride, uint64_t pw_stride) {
  if (l <= 0) return;
  if (l > kMaxQueries) throw ArgError("update_betas: too many queries");
  BStr t, u;
  t.s[0] = sizeof(ProofState);
  t.s[1] = pw_stride;
  u.s[0] = b_stride;
  u.s[1] = sizeof(ProofState);
  u.s[2] = pw_stride;
  if (batch == 1) t = u = BStr();
  ub_table_kernel<<<dim3(l, batch), 32, 0, s>>>(st, l, pw_scratch, t);
  GBZ_CUDA(cudaGetLastError());
  ub_kernel<<<dim3((unsigned)((nb + kUbSpan - 1) / kUbSpan), batch), kUbThreads, 0, s>>>(b, nb, st, l, pw_scratch, u);
  GBZ_CUDA(cudaGetLastError());
}

}  // namespace gbz
