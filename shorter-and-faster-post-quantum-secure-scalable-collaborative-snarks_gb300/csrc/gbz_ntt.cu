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
// Inside a pass every CTA holds B sub-transforms of length S in shared
// memory and runs self-sorting (Stockham) stages on them, radix 8 after one
// radix-2 or radix-4 stage when log2 S is not a multiple of 3.  The first
// stage runs on the values as they are loaded from global memory; the
// others read and write shared memory with __syncthreads between them.  The
// outer twiddle and the inverse scale are applied on the way out.  Groups of
// B >= 2 neighbouring columns make the strided pass read whole 32-byte
// sectors.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "gbz_internal.cuh"

namespace gbz {

namespace {

constexpr int kSubLog = 13;          // largest sub-transform held in shared memory
constexpr int kTwLoBits = 12;        // outer twiddle table split
constexpr int kMaxThreads = 1024;
constexpr int kCtaElems = 1 << kSubLog;  // most elements staged per CTA
constexpr int kPerThread = 8;            // elements per thread (CTA = max(32, E/8) threads)
constexpr int kLoadGroup = 4;            // global loads a thread issues back to back

// Four-step shape per length: the pass split (k1 = log2 of the contiguous
// pass B length) and the sub-transforms staged per CTA in each pass.  Set
// by ntt_set_shape (the autotuner) or derived by ntt_default_shape.
NttShape g_shape[kMaxLogN + 1];

struct PassArgs {
  const fe *in;
  fe *out;
  uint64_t n_valid;
  uint64_t in_gstride, in_jstride, out_gstride, out_kstride;
  const fe *wh;      // omega_{2^13}^t, t < 2^12 (first half), direction-specific
  const fe *tw_lo;   // omega_L^t, t < 2^12 (nullptr: no outer twiddle)
  const fe *tw_hi;   // omega_L^{2^12 t}
  const fe *tw_full; // pass A: omega_L^{n1 k2} at the output address n1 + N1 k2 (optional)
  fe scale;
  int logS, logB, has_scale, inverse;
  // Sparse rows (second pass of a sparse transform, the first pass folded
  // in): the input is sum_i sp_c[i] e_{q_i}, q_i = sp_q[i] >> sp_shift;
  // entries of one column (q mod the row length) are chained by sp_next
  // from the one flagged in sp_lead; sp_lo / sp_hi give omega_L^e and
  // sp_mask = L - 1.
  const int32_t *sp_q;
  const fe *sp_c;
  int sp_l, sp_shift;
  const int16_t *sp_next;
  const uint8_t *sp_lead;
  const fe *sp_lo, *sp_hi;
  uint64_t sp_mask;
  // Accumulating output: out[addr] += v for addr < acc_n, other outputs dropped.
  uint64_t acc_n;
  int acc;
  // Entries j >= j_valid of every sub-transform are zero (per-transform
  // padding of batched transforms; S when unused).
  uint32_t j_valid;
  // Independent transforms side by side: grid row y works on in + y row_in
  // and out + y row_out (0 for one transform).
  uint64_t row_in, row_out;
  // Packed real input: input entry j is (in[2j].re, in[2j+1].re) (two
  // base-field values as one extension element); a non-zero imaginary word
  // among them sets *nonreal.
  int pack_real;
  uint32_t *nonreal;
  // When set, the pass does nothing unless *run_if is non-zero.
  const uint32_t *run_if;
};

// Shared-memory swizzle: element a lives at a ^ ((a >> 3) & 7), which keeps
// both contiguous runs and stride-8 runs of 16-byte elements free of bank
// conflicts.
__device__ __forceinline__ uint32_t swz(uint32_t a) { return a ^ ((a >> 3) & 7u); }

// ---- lazy arithmetic inside one radix-8 butterfly -----------------------
// Values are kept below k*p (k <= 8 < 2^64 / p) and reduced once at the end.
// p - x for 0 <= x <= p is a bitwise complement within 61 bits.
__device__ __forceinline__ uint64_t lz_add(uint64_t a, uint64_t b) { return a + b; }
// a - b + m*p for b < m*p (m a power of two times p keeps it cheap: kp - b).
__device__ __forceinline__ uint64_t lz_sub(uint64_t a, uint64_t b, uint64_t mp) { return a + (mp - b); }
// Fold any 64-bit value to [0, p + 7] (p itself stands for zero).
__device__ __forceinline__ uint64_t fold(uint64_t x) { return (x & P) + (x >> 61); }
__device__ __forceinline__ uint64_t canon(uint64_t x) {  // [0, p + 7] -> [0, p)
  return x >= P ? x - P : x;
}
// A staged value (folded to [0, p + 7] by the last radix-8 stage, or
// canonical) made canonical for the output.
__device__ __forceinline__ fe canon_fe(fe x) { return fe_make(canon(x.re), canon(x.im)); }

struct lz {
  uint64_t re, im;
};
__device__ __forceinline__ lz lz_of(fe x) { return lz{x.re, x.im}; }
__device__ __forceinline__ lz lzadd(lz a, lz b) { return lz{lz_add(a.re, b.re), lz_add(a.im, b.im)}; }
__device__ __forceinline__ lz lzsub(lz a, lz b, uint64_t mp) { return lz{lz_sub(a.re, b.re, mp), lz_sub(a.im, b.im, mp)}; }

// Multiplications by the small roots on lazy values below 2p.
// getRootOfUnity(2) = -i and getRootOfUnity(3) = 2^30 (1 - i).
template <bool INV>
__device__ __forceinline__ lz lz_w4(lz x) {  // forward * (-i), inverse * i; input < 2p, output < 2p
  const uint64_t p2 = 2 * P;
  return INV ? lz{p2 - x.im, x.re} : lz{x.im, p2 - x.re};
}
// s * 2^30 (mod p) for s < 2^63: s = h 2^31 + l gives h 2^61 + l 2^30 = h + l 2^30;
// the result is below p + 2^32.
__device__ __forceinline__ uint64_t mul2e30(uint64_t s) { return ((s << 30) & P) + (s >> 31); }
// On inputs <= 2p per component the sums below stay within 4p; outputs < p + 2^32.
template <bool INV>
__device__ __forceinline__ lz lz_w8(lz x) {  // forward * 2^30 (1 - i), inverse * 2^30 (1 + i)
  const uint64_t s = mul2e30(x.re + x.im);
  const uint64_t d = INV ? mul2e30(x.re + (2 * P - x.im)) : mul2e30(x.im + (2 * P - x.re));
  return INV ? lz{d, s} : lz{s, d};
}
template <bool INV>
__device__ __forceinline__ lz lz_w8_3(lz x) {  // forward * 2^30 (-1 - i), inverse * 2^30 (-1 + i)
  const uint64_t ns = mul2e30(4 * P - (x.re + x.im));
  const uint64_t d = INV ? mul2e30(x.re + (2 * P - x.im)) : mul2e30(x.im + (2 * P - x.re));
  return INV ? lz{ns, d} : lz{d, ns};
}

// In-register DFTs with natural-order output: V[k] = sum_q v[q] w_R^{qk}.
// dft2 and dft4 take and return canonical values (they only run as the first
// stage); dft8 keeps its additions lazy (bounds at its definition).
template <bool INV>
__device__ __forceinline__ void dft2(fe *v) {
  fe a = v[0], b = v[1];
  v[0] = fadd(a, b);
  v[1] = fsub(a, b);
}
template <bool INV>
__device__ __forceinline__ void dft4(fe *v) {
  fe c0 = fadd(v[0], v[2]), c1 = fadd(v[1], v[3]);
  fe d0 = fsub(v[0], v[2]), d1 = fsub(v[1], v[3]);
  d1 = INV ? fe_make(subp(0, d1.im), d1.re) : fe_make(d1.im, subp(0, d1.re));
  v[0] = fadd(c0, c1);
  v[2] = fsub(c0, c1);
  v[1] = fadd(d0, d1);
  v[3] = fsub(d0, d1);
}
// Inputs: v[0] <= p + 7 (a folded output of the previous stage), v[1..7]
// <= p (canonical, or p standing for zero).  Every intermediate below stays
// within 8p + 7 = 2^64 - 1, and the outputs are folded once to [0, p + 7]:
// the next stage multiplies v[1..7] by twiddles (canonical products) and
// takes v[0] as it is; the pass epilogue makes the last stage's values
// canonical.
template <bool INV>
__device__ __forceinline__ void dft8(fe *v) {
  const uint64_t P2 = 2 * P, P4 = 4 * P;
  lz a[4], b[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {  // <= 2p (<= 2p + 7 for q = 0)
    a[q] = lzadd(lz_of(v[q]), lz_of(v[q + 4]));
    b[q] = lzsub(lz_of(v[q]), lz_of(v[q + 4]), P);
  }
  b[1] = lz_w8<INV>(b[1]);    // < p + 2^32
  b[2] = lz_w4<INV>(b[2]);    // <= 2p
  b[3] = lz_w8_3<INV>(b[3]);  // < p + 2^32
  // two radix-4 DFTs on inputs <= 2p (x[0] <= 2p + 7): c, d <= 4p + 7,
  // outputs <= 8p + 7
  lz out[8];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    lz *x = h ? b : a;
    lz c0 = lzadd(x[0], x[2]), c1 = lzadd(x[1], x[3]);
    lz d0 = lzsub(x[0], x[2], P2), d1 = lzsub(x[1], x[3], P2);
    // d1 * w4 on a value <= 4p: fold to <= p + 3 first
    d1 = lz{fold(d1.re), fold(d1.im)};
    d1 = INV ? lz{P2 - d1.im, d1.re} : lz{d1.im, P2 - d1.re};  // < 2p
    out[h + 0] = lzadd(c0, c1);       // V[0 + h]
    out[h + 4] = lzsub(c0, c1, P4);   // V[4 + h]
    out[h + 2] = lzadd(d0, d1);       // V[2 + h]
    out[h + 6] = lzsub(d0, d1, P4);   // V[6 + h]
  }
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = fe_make(fold(out[k].re), fold(out[k].im));
}

// omega_S^e from the half table T[t] = omega_S^t (t < S/2):
// omega_S^{t + S/2} = -omega_S^t.
__device__ __forceinline__ fe twiddle(const fe *T, uint32_t e, int logS) {
  const uint32_t hshift = logS - 1;
  const fe w = T[e & ((1u << hshift) - 1)];
  if (e >> hshift) return fe_make(w.re ? P - w.re : 0, w.im ? P - w.im : 0);
  return w;
}

// One radix-R Stockham stage over E staged elements (B sub-transforms of
// length S = 2^LOGS), Ns = 2^LOGNS = product of the earlier radices:
//   butterfly (b, j): v[r] = x[j + r S/R] * omega_{Ns R}^{r (j mod Ns)},
//   DFT_R(v), x'[(j/Ns) Ns R + (j mod Ns) + r Ns] = v[r].
// S and Ns are compile-time, so shifts, masks and the swizzled offsets of a
// butterfly's elements fold into immediates: when the stride between them is
// a multiple of 64 elements, swz(a + r stride) = swz(a) + r stride.
template <int R, bool INV, int LOGS, int LOGNS>
__device__ __forceinline__ void stockham_stage(fe *sm, const fe *T, int logE) {
  constexpr int LOGR = R == 8 ? 3 : (R == 4 ? 2 : 1);
  constexpr int PER = kPerThread / R;
  constexpr int logSR = LOGS - LOGR;
  const uint32_t nb = 1u << (logE - LOGR);
  fe v[PER * R];
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const uint32_t u = threadIdx.x + i * blockDim.x;
    if (u < nb) {
      const uint32_t b = u >> logSR, j = u & ((1u << logSR) - 1);
      const uint32_t base = (b << LOGS) + j;
      if constexpr (logSR >= 6) {
        const fe *src = sm + swz(base);
#pragma unroll
        for (int r = 0; r < R; r++) v[i * R + r] = src[(uint32_t)r << logSR];
      } else {
#pragma unroll
        for (int r = 0; r < R; r++) v[i * R + r] = sm[swz(base + ((uint32_t)r << logSR))];
      }
      if (LOGNS > 0) {
        const uint32_t k = j & ((1u << LOGNS) - 1);
        constexpr int sh = LOGS - LOGNS - LOGR;
        if (R == 8) {
          // k << sh < S/8, so the exponents r (k << sh) of r <= 4 stay in the
          // half table and only r = 5..7 may need the negation.
          const fe *tw = T + (k << sh);
          constexpr uint32_t half = 1u << (LOGS - 1);
#pragma unroll
          for (int r = 1; r <= 4; r++) v[i * R + r] = fmul(v[i * R + r], tw[(r - 1) * (k << sh)]);  // T[r (k << sh)]
#pragma unroll
          for (int r = 5; r < 8; r++) {
            const uint32_t e = r * (k << sh);
            const bool hi = e >= half;
            const fe w = T[hi ? e - half : e];
            v[i * R + r] = fmul(v[i * R + r], hi ? fe_make(P - w.re, P - w.im) : w);
          }
        } else {
#pragma unroll
          for (int r = 1; r < R; r++) v[i * R + r] = fmul(v[i * R + r], twiddle(T, (r * k) << sh, LOGS));
        }
      }
      if (R == 8) dft8<INV>(&v[i * R]);
      else if (R == 4) dft4<INV>(&v[i * R]);
      else dft2<INV>(&v[i * R]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const uint32_t u = threadIdx.x + i * blockDim.x;
    if (u < nb) {
      const uint32_t b = u >> logSR, j = u & ((1u << logSR) - 1);
      const uint32_t k = j & ((1u << LOGNS) - 1);
      const uint32_t dst = (b << LOGS) + ((j >> LOGNS) << (LOGNS + LOGR)) + k;
      if constexpr (LOGNS >= 6) {
        fe *d = sm + swz(dst);
#pragma unroll
        for (int r = 0; r < R; r++) d[(uint32_t)r << LOGNS] = v[i * R + r];
      } else {
#pragma unroll
        for (int r = 0; r < R; r++) sm[swz(dst + ((uint32_t)r << LOGNS))] = v[i * R + r];
      }
    }
  }
  __syncthreads();
}

template <bool INV, int LOGS, int LOGNS>
__device__ __forceinline__ void stockham_radix8(fe *sm, const fe *T, int logE) {
  if constexpr (LOGNS < LOGS) {
    stockham_stage<8, INV, LOGS, LOGNS>(sm, T, logE);
    stockham_radix8<INV, LOGS, LOGNS + 3>(sm, T, logE);
  }
}

// The stages of a length-2^LOGS transform: a radix-2 or radix-4 stage when
// LOGS is not a multiple of 3, then radix-8 stages.
template <bool INV, int LOGS>
__device__ __forceinline__ void stockham(fe *sm, const fe *T, int logE) {
  if constexpr (LOGS % 3 == 1) {
    stockham_stage<2, INV, LOGS, 0>(sm, T, logE);
    stockham_radix8<INV, LOGS, 1>(sm, T, logE);
  } else if constexpr (LOGS % 3 == 2) {
    stockham_stage<4, INV, LOGS, 0>(sm, T, logE);
    stockham_radix8<INV, LOGS, 2>(sm, T, logE);
  } else {
    stockham_radix8<INV, LOGS, 0>(sm, T, logE);
  }
}

template <bool INV>
__device__ __forceinline__ void stockham_dispatch(fe *sm, const fe *T, int logS, int logE) {
  switch (logS) {
    case 1: stockham<INV, 1>(sm, T, logE); break;
    case 2: stockham<INV, 2>(sm, T, logE); break;
    case 3: stockham<INV, 3>(sm, T, logE); break;
    case 4: stockham<INV, 4>(sm, T, logE); break;
    case 5: stockham<INV, 5>(sm, T, logE); break;
    case 6: stockham<INV, 6>(sm, T, logE); break;
    case 7: stockham<INV, 7>(sm, T, logE); break;
    case 8: stockham<INV, 8>(sm, T, logE); break;
    case 9: stockham<INV, 9>(sm, T, logE); break;
    case 10: stockham<INV, 10>(sm, T, logE); break;
    case 11: stockham<INV, 11>(sm, T, logE); break;
    case 12: stockham<INV, 12>(sm, T, logE); break;
    case 13: stockham<INV, 13>(sm, T, logE); break;
    default: break;  // length 1: nothing to do
  }
}

// The first stage (Ns = 1, no twiddles) fused into the staging from global
// memory: a thread loads the R inputs x[b, j + r S/R] of its butterflies,
// transforms them in registers and stores x'[b, R j + r], so the stage costs
// no shared-memory round trip.  Contiguous sub-transforms give consecutive
// threads consecutive j; strided ones (columns of the first four-step pass)
// consecutive sub-transforms b, whose columns are adjacent in memory.
template <bool INV, int LOGS, bool PACK>
__device__ __forceinline__ void staged_first_stage(fe *sm, const PassArgs &a, uint64_t g0, int logB, int logE) {
  constexpr int LOGR = LOGS % 3 == 1 ? 1 : (LOGS % 3 == 2 ? 2 : 3);
  constexpr int R = 1 << LOGR, PER = kPerThread / R, logSR = LOGS - LOGR;
  const uint32_t nb = 1u << (logE - LOGR);
  const bool contiguous = a.in_jstride == 1;
  fe v[PER][R];
  uint64_t nonreal = 0;
#pragma unroll
  for (int i = 0; i < PER; i++) {  // all loads first: PER * R = 8 in flight
    const uint32_t u = threadIdx.x + i * blockDim.x;
    const uint32_t b = contiguous ? u >> logSR : u & ((1u << logB) - 1);
    const uint32_t j = contiguous ? u & ((1u << logSR) - 1) : u >> logB;
    const uint64_t row = (g0 + b) * a.in_gstride;
#pragma unroll
    for (int r = 0; r < R; r++) {
      const uint32_t jj = j + ((uint32_t)r << logSR);
      const uint64_t addr = row + (uint64_t)jj * a.in_jstride;
      const bool ok = u < nb && addr < a.n_valid && jj < a.j_valid;
      if (!PACK) {
        v[i][r] = ok ? a.in[addr] : fe_zero();
      } else {
        const fe e0 = ok ? a.in[2 * addr] : fe_zero(), e1 = ok ? a.in[2 * addr + 1] : fe_zero();
        nonreal |= e0.im | e1.im;
        v[i][r] = fe_make(e0.re, e1.re);
      }
    }
  }
  if (PACK && nonreal) atomicOr(a.nonreal, 1u);
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const uint32_t u = threadIdx.x + i * blockDim.x;
    if (u < nb) {
      const uint32_t b = contiguous ? u >> logSR : u & ((1u << logB) - 1);
      const uint32_t j = contiguous ? u & ((1u << logSR) - 1) : u >> logB;
      if (R == 8) dft8<INV>(v[i]);
      else if (R == 4) dft4<INV>(v[i]);
      else dft2<INV>(v[i]);
      const uint32_t dst = (b << LOGS) + (j << LOGR);
#pragma unroll
      for (int r = 0; r < R; r++) sm[swz(dst + r)] = v[i][r];
    }
  }
}

template <bool INV, int LOGS, bool PACK>
__device__ __forceinline__ void staged_transform(fe *sm, const fe *T, const PassArgs &a, uint64_t g0, int logB,
                                                 int logE) {
  constexpr int LOGR = LOGS % 3 == 1 ? 1 : (LOGS % 3 == 2 ? 2 : 3);
  staged_first_stage<INV, LOGS, PACK>(sm, a, g0, logB, logE);
  __syncthreads();
  stockham_radix8<INV, LOGS, LOGR>(sm, T, logE);
}

template <bool INV, bool PACK>
__device__ __forceinline__ void staged_dispatch(fe *sm, const fe *T, const PassArgs &a, uint64_t g0, int logS,
                                                int logB, int logE) {
  switch (logS) {
    case 1: staged_transform<INV, 1, PACK>(sm, T, a, g0, logB, logE); break;
    case 2: staged_transform<INV, 2, PACK>(sm, T, a, g0, logB, logE); break;
    case 3: staged_transform<INV, 3, PACK>(sm, T, a, g0, logB, logE); break;
    case 4: staged_transform<INV, 4, PACK>(sm, T, a, g0, logB, logE); break;
    case 5: staged_transform<INV, 5, PACK>(sm, T, a, g0, logB, logE); break;
    case 6: staged_transform<INV, 6, PACK>(sm, T, a, g0, logB, logE); break;
    case 7: staged_transform<INV, 7, PACK>(sm, T, a, g0, logB, logE); break;
    case 8: staged_transform<INV, 8, PACK>(sm, T, a, g0, logB, logE); break;
    case 9: staged_transform<INV, 9, PACK>(sm, T, a, g0, logB, logE); break;
    case 10: staged_transform<INV, 10, PACK>(sm, T, a, g0, logB, logE); break;
    case 11: staged_transform<INV, 11, PACK>(sm, T, a, g0, logB, logE); break;
    case 12: staged_transform<INV, 12, PACK>(sm, T, a, g0, logB, logE); break;
    case 13: staged_transform<INV, 13, PACK>(sm, T, a, g0, logB, logE); break;
    default: break;
  }
}

// PACK: the first pass of a packed real transform (a separate instantiation,
// so that the general kernel keeps its register allocation).
template <bool PACK>
__global__ void __launch_bounds__(kMaxThreads) ntt_pass_kernel(PassArgs a) {
  if (a.run_if && *a.run_if == 0) return;  // uniform over the grid
  extern __shared__ fe smem[];
  a.in += blockIdx.y * a.row_in;
  a.out += blockIdx.y * a.row_out;
  const int logS = a.logS, logB = a.logB, logE = logS + logB;
  const uint32_t S = 1u << logS, total = 1u << logE;
  fe *sm = smem;
  fe *T = smem + total;  // S/2 twiddles omega_S^t
  const uint64_t g0 = (uint64_t)blockIdx.x << logB;

  if (logS >= 1) {
    const uint32_t nT = S >> 1;
    for (uint32_t t = threadIdx.x; t < nT; t += blockDim.x) T[t] = a.wh[t << (kSubLog - logS)];
  }
  if (a.sp_l > 0) {
    // Sparse rows: row k2 of the intermediate holds, in column n1, the sum
    // over the entries q = n1 (mod row length) of c * omega_L^{q k2}: the
    // first pass's column transform of a few nonzeros times its outer
    // twiddle, formed directly, so the first pass and its intermediate
    // array are skipped.  One thread per (first entry of a column, row).
    for (uint32_t e = threadIdx.x; e < total; e += blockDim.x) sm[e] = fe_zero();
    __syncthreads();
    const uint32_t l = (uint32_t)a.sp_l;
    for (uint32_t t = threadIdx.x; t < (l << logB); t += blockDim.x) {
      const uint32_t i = t % l, b = t / l;
      if (!a.sp_lead[i]) continue;
      const uint64_t k2 = g0 + b;
      fe v = fe_zero();
      int u = (int)i;
      for (uint32_t it = 0; it < l && u >= 0; it++, u = a.sp_next[u]) {
        const uint64_t q = (uint64_t)((uint32_t)a.sp_q[u] >> a.sp_shift);
        const uint64_t ex = (q * k2) & a.sp_mask;
        v = fadd(v, fmul(a.sp_c[u], fmul(a.sp_lo[ex & ((1u << kTwLoBits) - 1)], a.sp_hi[ex >> kTwLoBits])));
      }
      const uint32_t n1 = ((uint32_t)a.sp_q[i] >> a.sp_shift) & (S - 1);
      sm[swz((b << logS) + n1)] = v;
    }
    __syncthreads();
    if (a.inverse) stockham_dispatch<true>(sm, T, logS, logE);
    else stockham_dispatch<false>(sm, T, logS, logE);
  } else if (logS >= 1) {
    if (a.inverse) staged_dispatch<true, PACK>(sm, T, a, g0, logS, logB, logE);
    else staged_dispatch<false, PACK>(sm, T, a, g0, logS, logB, logE);
  } else {
    // Sub-transforms of length 1: staging only.
    // A thread stages at most kPerThread elements (blockDim >= total / 8);
    // groups of kLoadGroup loads are issued before their shared-memory
    // stores so that several global loads are in flight per thread.
    if (a.in_jstride == 1) {
      for (int i0 = 0; i0 < kPerThread; i0 += kLoadGroup) {
        fe v[kLoadGroup];
#pragma unroll
        for (int i = 0; i < kLoadGroup; i++) {
          const uint32_t e = threadIdx.x + (i0 + i) * blockDim.x;
          const uint32_t b = e >> logS, j = e & (S - 1);
          const uint64_t addr = (g0 + b) * a.in_gstride + j;
          v[i] = (e < total && addr < a.n_valid && j < a.j_valid) ? a.in[addr] : fe_zero();
        }
#pragma unroll
        for (int i = 0; i < kLoadGroup; i++) {
          const uint32_t e = threadIdx.x + (i0 + i) * blockDim.x;
          if (e < total) sm[swz(e)] = v[i];
        }
      }
    } else {
      for (int i0 = 0; i0 < kPerThread; i0 += kLoadGroup) {
        fe v[kLoadGroup];
#pragma unroll
        for (int i = 0; i < kLoadGroup; i++) {
          const uint32_t e = threadIdx.x + (i0 + i) * blockDim.x;
          const uint32_t b = e & ((1u << logB) - 1), j = e >> logB;
          const uint64_t addr = (g0 + b) * a.in_gstride + (uint64_t)j * a.in_jstride;
          v[i] = (e < total && addr < a.n_valid && j < a.j_valid) ? a.in[addr] : fe_zero();
        }
#pragma unroll
        for (int i = 0; i < kLoadGroup; i++) {
          const uint32_t e = threadIdx.x + (i0 + i) * blockDim.x;
          const uint32_t b = e & ((1u << logB) - 1), j = e >> logB;
          if (e < total) sm[swz((b << logS) + j)] = v[i];
        }
      }
    }
    __syncthreads();
  }

  if (a.out_kstride == 1) {
    for (uint32_t e = threadIdx.x; e < total; e += blockDim.x) {
      const uint32_t b = e >> logS, k = e & (S - 1);
      fe v = canon_fe(sm[swz(e)]);
      if (a.tw_lo) {
        const uint64_t ex = (g0 + b) * k;
        v = fmul(v, fmul(a.tw_lo[ex & ((1u << kTwLoBits) - 1)], a.tw_hi[ex >> kTwLoBits]));
      }
      if (a.has_scale) v = fmul(v, a.scale);
      const uint64_t addr = (g0 + b) * a.out_gstride + k;
      if (!a.acc) a.out[addr] = v;
      else if (addr < a.acc_n) a.out[addr] = fadd(a.out[addr], v);
    }
  } else if (a.tw_full && !a.has_scale && !a.acc) {
    // first pass with the full twiddle table: issue each group's table
    // loads before its multiplies
    for (int i0 = 0; i0 < kPerThread; i0 += kLoadGroup) {
      fe tw[kLoadGroup];
#pragma unroll
      for (int i = 0; i < kLoadGroup; i++) {
        const uint32_t e = threadIdx.x + (i0 + i) * blockDim.x;
        const uint32_t b = e & ((1u << logB) - 1), k = e >> logB;
        const uint64_t addr = (g0 + b) * a.out_gstride + (uint64_t)k * a.out_kstride;
        tw[i] = e < total ? a.tw_full[addr] : fe_zero();
      }
#pragma unroll
      for (int i = 0; i < kLoadGroup; i++) {
        const uint32_t e = threadIdx.x + (i0 + i) * blockDim.x;
        if (e >= total) continue;
        const uint32_t b = e & ((1u << logB) - 1), k = e >> logB;
        const uint64_t addr = (g0 + b) * a.out_gstride + (uint64_t)k * a.out_kstride;
        a.out[addr] = fmul(sm[swz((b << logS) + k)], tw[i]);  // takes the folded value as it is
      }
    }
  } else {
    for (uint32_t e = threadIdx.x; e < total; e += blockDim.x) {
      const uint32_t b = e & ((1u << logB) - 1), k = e >> logB;
      fe v = canon_fe(sm[swz((b << logS) + k)]);
      const uint64_t addr = (g0 + b) * a.out_gstride + (uint64_t)k * a.out_kstride;
      if (a.tw_full) {
        v = fmul(v, a.tw_full[addr]);
      } else if (a.tw_lo) {
        const uint64_t ex = (g0 + b) * k;
        v = fmul(v, fmul(a.tw_lo[ex & ((1u << kTwLoBits) - 1)], a.tw_hi[ex >> kTwLoBits]));
      }
      if (a.has_scale) v = fmul(v, a.scale);
      if (!a.acc) a.out[addr] = v;
      else if (addr < a.acc_n) a.out[addr] = fadd(a.out[addr], v);
    }
  }
}

// First half of the omega_{2^13} powers, per direction; shared by every length.
fe *g_wq[2] = {nullptr, nullptr};
int g_wq_device = -1;
constexpr size_t kMaxSmem = sizeof(fe) * (kCtaElems + kCtaElems / 2);

void ensure_wq() {
  int dev;
  GBZ_CUDA(cudaGetDevice(&dev));
  if (g_wq[0] && g_wq_device == dev) return;
  const int n = 1 << (kSubLog - 1);
  std::vector<fe> h(n);
  for (int dir = 0; dir < 2; dir++) {
    fe w = root_of_unity(kSubLog);
    if (dir) w = finv(w);
    fe x = fe_one();
    for (int t = 0; t < n; t++) { h[t] = x; x = fmul(x, w); }
    GBZ_CUDA(cudaMalloc(&g_wq[dir], sizeof(fe) * n));
    GBZ_CUDA(cudaMemcpy(g_wq[dir], h.data(), sizeof(fe) * n, cudaMemcpyHostToDevice));
  }
  g_wq_device = dev;
  GBZ_CUDA(cudaFuncSetAttribute(ntt_pass_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
  GBZ_CUDA(cudaFuncSetAttribute(ntt_pass_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
}

// Column chains of a sparse input: next[t] = the next entry with the same
// column ((q >> shift) & colmask), -1 at the end; lead[t] = 1 for the first
// entry of each column.  One thread per entry (l <= kMaxQueries).
__global__ void sparse_chain_kernel(const int32_t *q, int l, int shift, uint32_t colmask, int16_t *next,
                                    uint8_t *lead) {
  __shared__ uint32_t col[kMaxQueries];
  const int t = threadIdx.x;
  if (t < l) col[t] = ((uint32_t)q[t] >> shift) & colmask;
  __syncthreads();
  if (t >= l) return;
  int nx = -1;
  uint8_t first = 1;
  for (int u = 0; u < l; u++) {
    if (col[u] != col[t]) continue;
    if (u < t) first = 0;
    else if (u > t && nx < 0) nx = u;
  }
  next[t] = (int16_t)nx;
  lead[t] = first;
}

void launch_pass(const PassArgs &a, uint64_t groups, cudaStream_t s, int rows = 1) {
  const uint64_t blocks = groups >> a.logB;
  const uint32_t E = 1u << (a.logS + a.logB);
  const size_t smem = sizeof(fe) * (E + (a.logS >= 1 ? (1u << (a.logS - 1)) : 0));
  const unsigned threads = E / kPerThread > 32 ? E / kPerThread : 32;
  if (rows < 1 || rows > 65535) throw ArgError("transform: 1..65535 rows per launch");
  if (a.pack_real) ntt_pass_kernel<true><<<dim3((unsigned)blocks, (unsigned)rows), threads, smem, s>>>(a);
  else ntt_pass_kernel<false><<<dim3((unsigned)blocks, (unsigned)rows), threads, smem, s>>>(a);
  GBZ_CUDA(cudaGetLastError());
}

}  // namespace

// Full outer-twiddle tables of the first pass, per (device, length, split,
// direction): T[n1 + N1 k2] = omega_L^{n1 k2}, so the pass multiplies once
// per element instead of forming the twiddle from the two-level table.
// The integer pipes bound the transform and HBM has room, so reading
// 16 B per element is the cheaper side of the trade.
std::mutex g_outer_mu;
std::map<std::tuple<int, int, int, int>, fe *> g_outer;
bool g_use_outer = true;  // gbz_ntt_full_twiddles

// T[n1 + N1 k] = w^(n1 k) for n1 < N1, k < N2: thread (n1, chunk) walks 64
// consecutive k from w^(n1 k0) by products with w^n1.
__global__ void outer_table_kernel(fe w, int logL, int k1, fe *T) {
  const uint64_t N1 = 1ull << k1, N2 = 1ull << (logL - k1);
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t chunks = (N2 + 63) / 64;
  if (tid >= N1 * chunks) return;
  const uint64_t n1 = tid % N1, k0 = (tid / N1) * 64;
  const fe wn1 = fpow(w, n1);
  fe x = fpow(wn1, k0);
  for (uint64_t k = k0; k < k0 + 64 && k < N2; k++) {
    T[n1 + N1 * k] = x;
    x = fmul(x, wn1);
  }
}

const fe *outer_table_get(int logn, int k1, bool inverse) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_outer_mu);
  auto it = g_outer.find(std::make_tuple(dev, logn, k1, inverse ? 1 : 0));
  return it == g_outer.end() ? nullptr : it->second;
}

void outer_table_build(int logn, int k1) {
  if (logn <= kSubLog || k1 < 1 || k1 >= logn) return;
  int dev = 0;
  GBZ_CUDA(cudaGetDevice(&dev));
  for (int dir = 0; dir < 2; dir++) {
    const auto key = std::make_tuple(dev, logn, k1, dir);
    {
      std::lock_guard<std::mutex> lk(g_outer_mu);
      if (g_outer.count(key)) continue;
    }
    const uint64_t L = 1ull << logn;
    fe *T = nullptr;
    if (cudaMalloc(&T, sizeof(fe) * L) != cudaSuccess) {
      cudaGetLastError();  // no room: the pass keeps the two-level twiddles
      return;
    }
    fe w = root_of_unity(logn);
    if (dir) w = finv(w);
    const uint64_t threads = (1ull << k1) * (((L >> k1) + 63) / 64);
    outer_table_kernel<<<(unsigned)((threads + 255) / 256), 256>>>(w, logn, k1, T);
    GBZ_CUDA(cudaGetLastError());
    GBZ_CUDA(cudaDeviceSynchronize());
    std::lock_guard<std::mutex> lk(g_outer_mu);
    g_outer[key] = T;
  }
}

// Frees the tables of other splits of this length (after autotuning).
void outer_table_keep_only(int logn, int k1) {
  int dev = 0;
  GBZ_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_outer_mu);
  for (auto it = g_outer.begin(); it != g_outer.end();) {
    if (std::get<0>(it->first) == dev && std::get<1>(it->first) == logn && std::get<2>(it->first) != k1) {
      GBZ_CUDA(cudaDeviceSynchronize());
      cudaFree(it->second);
      it = g_outer.erase(it);
    } else {
      ++it;
    }
  }
}

void ntt_use_full_twiddles(bool on) { g_use_outer = on; }

void ntt_tables_build(NttTables &t, int logn) {
  ensure_wq();
  t.logn = logn;
  t.sub_fwd = g_wq[0];
  t.sub_inv = g_wq[1];
  t.inv_len = finv(fe_make(1ull << logn, 0));
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
  if (logn > kSubLog) outer_table_build(logn, ntt_get_shape(logn).k1);
}

int ntt_launch_count(int logn) { return logn <= kSubLog ? 1 : 2; }

NttShape ntt_default_shape(int logn) {
  NttShape sh;
  sh.k1 = (logn + 1) / 2;
  const int k2 = logn - sh.k1;
  // Strided pass: at least two neighbouring columns per CTA (whole 32-byte
  // sectors) and up to 2^13 staged elements, fewer when the transform is
  // small so that it still spreads over many CTAs.
  sh.logBA = std::min(sh.k1, std::max(k2 < kSubLog ? 1 : 0, std::min(kSubLog, logn - 8) - k2));
  sh.logBB = std::min(k2, std::max(0, std::min(kSubLog - 1, logn - 8) - sh.k1));
  return sh;
}

bool ntt_shape_valid(int logn, const NttShape &sh) {
  if (logn <= kSubLog || logn > kMaxNttLogN) return false;
  const int k2 = logn - sh.k1;
  if (sh.k1 < 1 || sh.k1 > kSubLog || k2 < 1 || k2 > kSubLog) return false;
  if (sh.logBA < 0 || sh.logBA > sh.k1 || k2 + sh.logBA > kSubLog) return false;
  if (sh.logBB < 0 || sh.logBB > k2 || sh.k1 + sh.logBB > kSubLog) return false;
  return true;
}

NttShape ntt_get_shape(int logn) {
  if (logn <= kSubLog || logn > kMaxNttLogN) return NttShape{};
  return g_shape[logn].k1 > 0 ? g_shape[logn] : ntt_default_shape(logn);
}

void ntt_set_shape(int logn, const NttShape &sh) {
  if (!ntt_shape_valid(logn, sh)) throw ArgError("ntt shape: invalid split or staging for this length");
  outer_table_build(logn, sh.k1);
  g_shape[logn] = sh;
}

std::vector<NttShape> ntt_shape_candidates(int logn) {
  std::vector<NttShape> out;
  for (int k1 = 1; k1 <= kSubLog; k1++) {
    const int k2 = logn - k1;
    if (k2 < 1 || k2 > kSubLog || std::abs(k1 - k2) > 2) continue;
    for (int a = 0; a <= std::min(k1, kSubLog - k2); a++)
      for (int b = 0; b <= std::min(k2, kSubLog - k1); b++) {
        NttShape sh{k1, a, b};
        if ((a == 0 && k2 < kSubLog) || a > 4 || b > 3) continue;  // keep sector-sized column groups
        if (ntt_shape_valid(logn, sh)) out.push_back(sh);
      }
  }
  return out;
}

void ntt_tables_free(NttTables &t) {
  cudaFree(t.lo_fwd);
  cudaFree(t.hi_fwd);
  cudaFree(t.lo_inv);
  cudaFree(t.hi_inv);
  t.lo_fwd = t.hi_fwd = t.lo_inv = t.hi_inv = nullptr;
  t.logn = -1;
}

namespace {

// Shared by the dense transform and the sparse/accumulating variant.
// Options of a transform: packed real input (the pass that reads `in`) and
// a device flag that gates every pass.
struct PassGate {
  int pack_real = 0;
  uint32_t *nonreal = nullptr;
  const uint32_t *run_if = nullptr;
};

void ntt_two_pass(const NttTables &t, const fe *in, uint64_t n_valid, fe *out, fe *tmp, bool inverse,
                  cudaStream_t s, int rows = 1, uint64_t row_in = 0, uint64_t row_out = 0,
                  const PassGate &gate = PassGate(), uint64_t out_elem_stride = 1) {
  const int logn = t.logn;
  const uint64_t L = 1ull << logn;
  if (logn > kMaxNttLogN) throw ArgError("transform longer than 2^26 (two passes of at most 2^13)");
  if (gate.pack_real && (logn < 1 || rows != 1)) throw ArgError("packed real transform: one row, length >= 2");
  if (n_valid > L) n_valid = L;
  PassArgs a{};
  a.pack_real = gate.pack_real;
  a.nonreal = gate.nonreal;
  a.run_if = gate.run_if;
  a.row_in = row_in;
  a.row_out = row_out;
  a.wh = inverse ? t.sub_inv : t.sub_fwd;
  a.scale = t.inv_len;
  a.inverse = inverse ? 1 : 0;
  a.j_valid = 1u << kSubLog;
  if (logn <= kSubLog) {
    a.in = in;
    a.out = out;
    a.n_valid = n_valid;
    a.in_gstride = L;
    a.in_jstride = 1;
    a.out_gstride = L;
    a.out_kstride = out_elem_stride;
    a.logS = logn;
    a.logB = 0;
    a.has_scale = inverse;
    a.tw_lo = nullptr;
    a.tw_hi = nullptr;
    launch_pass(a, 1, s, rows);
    return;
  }
  const NttShape sh = g_shape[logn].k1 > 0 ? g_shape[logn] : ntt_default_shape(logn);
  const int k1 = sh.k1;       // pass B (contiguous rows)
  const int k2 = logn - k1;   // pass A (strided columns)
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
  // Strided pass: at least two neighbouring columns per CTA (whole 32-byte
  // sectors) and up to 2^13 staged elements, fewer when the transform is
  // small so that it still spreads over many CTAs.
  a.logB = sh.logBA;
  a.tw_lo = inverse ? t.lo_inv : t.lo_fwd;
  a.tw_hi = inverse ? t.hi_inv : t.hi_fwd;
  a.tw_full = g_use_outer ? outer_table_get(logn, k1, inverse) : nullptr;
  a.has_scale = 0;
  a.row_out = L;  // the intermediate holds one full row per transform
  launch_pass(a, N1, s, rows);
  // pass B: rows k2 < N2, length N1, contiguous
  PassArgs b = a;
  b.pack_real = 0;  // only the first pass reads the input
  b.in = tmp;
  b.out = out;
  b.n_valid = L;
  b.in_gstride = N1;
  b.in_jstride = 1;
  b.out_gstride = out_elem_stride;
  b.out_kstride = N2 * out_elem_stride;
  b.logS = k1;
  b.logB = sh.logBB;
  b.tw_lo = nullptr;
  b.tw_hi = nullptr;
  b.tw_full = nullptr;
  b.has_scale = inverse;
  b.row_in = L;
  b.row_out = row_out;
  launch_pass(b, N2, s, rows);
}

}  // namespace

void ntt_launch(const NttTables &t, const fe *in, uint64_t n_valid, fe *out, fe *tmp, bool inverse,
                cudaStream_t s) {
  ntt_two_pass(t, in, n_valid, out, tmp, inverse, s);
}

namespace {
// x / 2 mod p for canonical x: 2 is invertible and x + p is even when x is odd.
__device__ __forceinline__ uint64_t half_p(uint64_t x) { return (x + ((x & 1) ? P : 0)) >> 1; }
__device__ __forceinline__ fe conj_fe(fe x) { return fe_make(x.re, x.im ? P - x.im : 0); }

// Real-input transform, last step.  Z = DFT_M(z), z_j = x_2j + i x_2j+1
// (M = N/2, omega_M = omega_N^2).  In F_{p^2} conjugation is the Frobenius
// x -> x^p and p = -1 mod N, so conj(omega_N) = omega_N^{-1}; for base-field
// x this gives E[k] = (Z[k] + conj Z[M-k]) / 2 = DFT_M(x_even)[k] and
// O[k] = (Z[k] - conj Z[M-k]) / 2i = DFT_M(x_odd)[k], then X[k] = E + w^k O,
// X[k+M] = E - w^k O (w = omega_N), and X[N-k] = conj X[k].  Thread t takes
// k = t and M - t (t = 0 and t = M/2 alone): 2 reads, 4 writes, 2 multiplies.
__global__ void real_unpack_kernel(const fe *__restrict__ Z, uint64_t M, const fe *lo, const fe *hi,
                                   fe *__restrict__ X) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t > M / 2) return;
  const fe a = Z[t], b = Z[t == 0 ? 0 : M - t];
  const fe E = fe_make(half_p(addp(a.re, b.re)), half_p(subp(a.im, b.im)));
  const fe O = fe_make(half_p(addp(a.im, b.im)), half_p(subp(b.re, a.re)));
  const fe w = fmul(lo[t & ((1u << kTwLoBits) - 1)], hi[t >> kTwLoBits]);
  const fe wo = fmul(w, O);
  const fe xk = fadd(E, wo), xkm = fsub(E, wo);
  X[t] = xk;
  X[t + M] = xkm;
  if (t != 0 && t != M / 2) {
    X[M - t] = conj_fe(xkm);
    X[2 * M - t] = conj_fe(xk);
  }
}
}  // namespace

void ntt_launch_real(const NttTables &t_half, const NttTables &t_full, const fe *in, uint64_t n_valid, fe *out,
                     fe *tmp, uint32_t *nonreal, cudaStream_t s) {
  const int logn = t_full.logn;
  if (t_half.logn != logn - 1 || logn < 2) throw ArgError("real transform: tables of lengths N/2 and N, N >= 4");
  if (n_valid & 1) throw ArgError("real transform: even number of input entries");
  const uint64_t N = 1ull << logn, M = N / 2;
  fe *Z = tmp + M;  // tmp holds N entries: the half-length intermediate, then Z
  PassGate g;
  g.pack_real = 1;
  g.nonreal = nonreal;
  ntt_two_pass(t_half, in, n_valid / 2, Z, tmp, false, s, 1, 0, 0, g);
  const uint64_t threads = M / 2 + 1;
  real_unpack_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(Z, M, t_full.lo_fwd, t_full.hi_fwd, out);
  GBZ_CUDA(cudaGetLastError());
  // any imaginary word: the general transform replaces the result
  PassGate f;
  f.run_if = nonreal;
  ntt_two_pass(t_full, in, n_valid, out, tmp, false, s, 1, 0, 0, f);
}

int ntt_launch_real_count(int logn) { return ntt_launch_count(logn - 1) + 1 + ntt_launch_count(logn); }

void ntt_launch_rows(const NttTables &t, const fe *in, uint64_t n_valid, uint64_t in_stride, fe *out,
                     uint64_t out_stride, int rows, fe *tmp, bool inverse, cudaStream_t s, uint64_t out_elem_stride) {
  if (rows < 1) return;
  if (out_elem_stride < 1) throw ArgError("transform: output element stride >= 1");
  ntt_two_pass(t, in, n_valid, out, tmp, inverse, s, rows, in_stride, out_stride, PassGate(), out_elem_stride);
}

void ntt_batched(const NttTables &t, const fe *in, uint64_t in_stride, uint32_t j_valid, fe *out, uint64_t count,
                 bool inverse, cudaStream_t s) {
  const int logS = t.logn;
  if (logS > kSubLog) throw ArgError("batched transform longer than 2^13");
  if (!count) return;
  PassArgs a{};
  a.wh = inverse ? t.sub_inv : t.sub_fwd;
  a.scale = t.inv_len;
  a.inverse = inverse ? 1 : 0;
  a.in = in;
  a.out = out;
  a.n_valid = ~0ull;
  a.j_valid = j_valid;
  a.in_gstride = in_stride;
  a.in_jstride = 1;
  a.out_gstride = 1ull << logS;
  a.out_kstride = 1;
  a.logS = logS;
  a.has_scale = inverse;
  // up to 2^12 staged elements per CTA, never more transforms than there are
  int logB = std::max(0, 12 - logS);
  while (logB > 0 && (1ull << logB) > count) logB--;
  a.logB = logB;
  const uint64_t B = 1ull << logB;
  const uint64_t full = count / B * B;
  if (full) launch_pass(a, full, s);
  if (full < count) {  // remaining transforms one per CTA
    PassArgs r = a;
    r.in = in + full * in_stride;
    r.out = out + (full << logS);
    r.logB = 0;
    launch_pass(r, count - full, s);
  }
}

void ntt_batched_strided(const NttTables &t, const fe *in, uint64_t col_stride, uint32_t j_valid, fe *out,
                         uint64_t count, bool inverse, cudaStream_t s) {
  const int logS = t.logn;
  if (logS > kSubLog) throw ArgError("batched transform longer than 2^13");
  if (!count) return;
  PassArgs a{};
  a.wh = inverse ? t.sub_inv : t.sub_fwd;
  a.scale = t.inv_len;
  a.inverse = inverse ? 1 : 0;
  a.in = in;
  a.out = out;
  a.n_valid = ~0ull;
  a.j_valid = j_valid;
  a.in_gstride = 1;            // transform g starts at in[g]
  a.in_jstride = col_stride;   // its entry j at in[g + j * col_stride]
  a.out_gstride = 1ull << logS;
  a.out_kstride = 1;
  a.logS = logS;
  a.has_scale = inverse;
  // neighbouring transforms share 32-byte sectors: stage at least two per CTA
  int logB = std::max(0, 12 - logS);
  while (logB > 0 && (1ull << logB) > count) logB--;
  a.logB = logB;
  const uint64_t B = 1ull << logB;
  const uint64_t full = count / B * B;
  if (full) launch_pass(a, full, s);
  if (full < count) {
    PassArgs r = a;
    r.in = in + full;
    r.out = out + (full << logS);
    r.logB = 0;
    launch_pass(r, count - full, s);
  }
}

void ntt_sparse_accumulate(const NttTables &t, const int32_t *q, const fe *c, int l, fe *acc, uint64_t nacc,
                           fe *tmp, cudaStream_t s, int q_shift) {
  if (t.logn <= kSubLog) throw ArgError("sparse transform needs a two-pass length");
  if (q_shift < 0 || q_shift > 8) throw ArgError("sparse transform: position shift out of range");
  if (l < 1 || l > kMaxQueries) throw ArgError("sparse transform: 1..256 entries");
  const int logn = t.logn;
  const uint64_t L = 1ull << logn;
  const NttShape sh = g_shape[logn].k1 > 0 ? g_shape[logn] : ntt_default_shape(logn);
  const int k1 = sh.k1, k2 = logn - k1;
  const uint64_t N1 = 1ull << k1, N2 = 1ull << k2;
  // column chains in the (otherwise unused) scratch
  int16_t *next = reinterpret_cast<int16_t *>(tmp);
  uint8_t *lead = reinterpret_cast<uint8_t *>(next + kMaxQueries);
  sparse_chain_kernel<<<1, kMaxQueries, 0, s>>>(q, l, q_shift, (uint32_t)(N1 - 1), next, lead);
  GBZ_CUDA(cudaGetLastError());
  PassArgs b{};
  b.wh = t.sub_fwd;
  b.scale = t.inv_len;
  b.inverse = 0;
  b.j_valid = 1u << kSubLog;
  b.in = nullptr;
  b.out = acc;
  b.n_valid = L;
  b.in_gstride = N1;
  b.in_jstride = 1;
  b.out_gstride = 1;
  b.out_kstride = N2;
  b.logS = k1;
  b.logB = sh.logBB;
  b.has_scale = 0;
  b.acc = 1;
  b.acc_n = nacc;
  b.sp_q = q;
  b.sp_c = c;
  b.sp_l = l;
  b.sp_shift = q_shift;
  b.sp_next = next;
  b.sp_lead = lead;
  b.sp_lo = t.lo_fwd;
  b.sp_hi = t.hi_fwd;
  b.sp_mask = L - 1;
  launch_pass(b, N2, s);
}

}  // namespace gbz
