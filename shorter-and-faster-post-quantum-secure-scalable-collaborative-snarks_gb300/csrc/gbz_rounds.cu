// Round forms of the multilinear sumcheck provers and the device-resident
// distributed sumcheck (gbz_rounds.cuh).
//
// Every form sums, over the pairs (v[2j], v[2j+1]) of its vectors, a product
// of the lines l(x) = (v[2j+1] - v[2j]) x + v[2j] (linear_poly,
// polynomial.h:46-59), coefficients highest degree first:
//   quadratic (v1, v2)            sum l1 l2                    coSumcheck_MPI.cpp:199
//   cubic (v1, v2, v3)            sum l1 l2 l3                 Distributed_Sumcheck.cpp:1144-1151
//   batch (v1..v4, r1, r2; b)     sum l1 l2 + l3 l4 + b lr1 lr2 coSumcheck_MPI.cpp:156-176
//   zero-check (v1, v2, v3, beta, r1, r2; b)
//                                 sum (l1 l2 + b lr1 lr2 - x l3) lbeta   coSumcheck_MPI.cpp:12-32
//   quadruple (v1..v4)            sum l1 l2 l3 l4              delegate_protocol.cpp:66-76
// and folds every vector by the round challenge r: v[j] = v[2j] + r (v[2j+1]
// - v[2j]) (coSumcheck_MPI.cpp:34-44, 178-187).  The fold of round i and the
// message of round i + 1 are one pass (four entries of every vector per
// thread).  All arithmetic is exact, so the summation order does not change
// a single bit of the result.
#include "gbz_rounds.cuh"

namespace gbz {

namespace {

constexpr int kThreads = 256;

template <int FORM> struct Form;
template <> struct Form<SC_QUADRATIC> { static constexpr int NV = 2, NC = 3; };
template <> struct Form<SC_CUBIC> { static constexpr int NV = 3, NC = 4; };
template <> struct Form<SC_BATCH> { static constexpr int NV = 6, NC = 3; };
template <> struct Form<SC_ZEROCHECK> { static constexpr int NV = 6, NC = 4; };
template <> struct Form<SC_QUADRUPLE> { static constexpr int NV = 4, NC = 5; };

struct Line {
  fe a, b, h;  // a x + b, h = a + b (the value at 1)
};
__device__ __forceinline__ Line line(fe lo, fe hi) { return Line{fsub(hi, lo), lo, hi}; }

// x / 2 in F_p: (x + p x_0) / 2 of each word.
__device__ __forceinline__ uint64_t halfp(uint64_t x) { return (x & 1) ? (x + P) >> 1 : x >> 1; }
__device__ __forceinline__ fe fhalf(fe x) { return fe_make(halfp(x.re), halfp(x.im)); }

// The cubic form accumulates, per thread, the sums of its products at 0, 1,
// -1 and the leading coefficient (8 products a pair instead of 9); this
// turns them into the coefficients (x^3, x^2, x, 1) before the sums are
// combined across threads.  The map is linear and exact, so the messages
// are the coefficient sums the reference forms pair by pair.
template <int FORM>
__device__ __forceinline__ void acc_to_coeffs(fe *acc) {
  if (FORM == SC_CUBIC) {
    const fe e_inf = acc[0], e1 = acc[1], em = acc[2], e0 = acc[3];
    acc[1] = fsub(fhalf(fadd(e1, em)), e0);     // c(1) + c(-1) = 2 (c2 + c0)
    acc[2] = fsub(fhalf(fsub(e1, em)), e_inf);  // c(1) - c(-1) = 2 (c3 + c1)
  }
}

// (a1 x + b1)(a2 x + b2) with three products
__device__ __forceinline__ void lmul(const Line &x, const Line &y, fe q[3]) {
  q[0] = fmul(x.a, y.a);
  q[2] = fmul(x.b, y.b);
  q[1] = fsub(fsub(fmul(fadd(x.a, x.b), fadd(y.a, y.b)), q[0]), q[2]);
}
// (q0 x^2 + q1 x + q2)(a x + b)
__device__ __forceinline__ void qlmul(const fe q[3], const Line &l, fe c[4]) {
  c[0] = fmul(q[0], l.a);
  c[1] = fadd(fmul(q[0], l.b), fmul(q[1], l.a));
  c[2] = fadd(fmul(q[1], l.b), fmul(q[2], l.a));
  c[3] = fmul(q[2], l.b);
}

template <int FORM>
__device__ __forceinline__ void accumulate(const Line *l, fe b, fe *acc) {
  fe q[3], c[4];
  if (FORM == SC_QUADRATIC) {
    lmul(l[0], l[1], q);
    for (int k = 0; k < 3; k++) acc[k] = fadd(acc[k], q[k]);
  } else if (FORM == SC_CUBIC) {
    // leading coefficient, values at 1, -1 (b - a) and 0 (acc_to_coeffs)
    const fe m0 = fsub(l[0].b, l[0].a), m1 = fsub(l[1].b, l[1].a), m2 = fsub(l[2].b, l[2].a);
    acc[0] = fadd(acc[0], fmul(fmul(l[0].a, l[1].a), l[2].a));
    acc[1] = fadd(acc[1], fmul(fmul(l[0].h, l[1].h), l[2].h));
    acc[2] = fadd(acc[2], fmul(fmul(m0, m1), m2));
    acc[3] = fadd(acc[3], fmul(fmul(l[0].b, l[1].b), l[2].b));
  } else if (FORM == SC_QUADRUPLE) {
    // ((l1 l2) l3) l4 as the reference multiplies them (polynomial.cpp:91-101)
    lmul(l[0], l[1], q);
    qlmul(q, l[2], c);
    acc[0] = fadd(acc[0], fmul(c[0], l[3].a));
    acc[1] = fadd(acc[1], fadd(fmul(c[1], l[3].a), fmul(c[0], l[3].b)));
    acc[2] = fadd(acc[2], fadd(fmul(c[2], l[3].a), fmul(c[1], l[3].b)));
    acc[3] = fadd(acc[3], fadd(fmul(c[3], l[3].a), fmul(c[2], l[3].b)));
    acc[4] = fadd(acc[4], fmul(c[3], l[3].b));
  } else if (FORM == SC_BATCH) {
    fe q2[3], qr[3];
    lmul(l[0], l[1], q);
    lmul(l[2], l[3], q2);
    lmul(l[4], l[5], qr);
    for (int k = 0; k < 3; k++) acc[k] = fadd(acc[k], fadd(fadd(q[k], q2[k]), fmul(b, qr[k])));
  } else {
    fe qr[3];
    lmul(l[0], l[1], q);
    lmul(l[4], l[5], qr);
    q[0] = fadd(q[0], fmul(b, qr[0]));
    q[1] = fsub(fadd(q[1], fmul(b, qr[1])), l[2].a);
    q[2] = fsub(fadd(q[2], fmul(b, qr[2])), l[2].b);
    qlmul(q, l[3], c);
    for (int k = 0; k < 4; k++) acc[k] = fadd(acc[k], c[k]);
  }
}

__device__ __forceinline__ fe shfl_down_fe(fe v, int d) {
  fe r;
  r.re = __shfl_down_sync(0xffffffffu, v.re, d);
  r.im = __shfl_down_sync(0xffffffffu, v.im, d);
  return r;
}

// Block sum of NC field elements; valid in thread 0.
template <int NC>
__device__ void block_sum(fe *x) {
  __shared__ fe red[kMaxFormCoeffs][kThreads / 32];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1)
#pragma unroll
    for (int k = 0; k < NC; k++) x[k] = fadd(x[k], shfl_down_fe(x[k], d));
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int k = 0; k < NC; k++) red[k][w] = x[k];
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    for (int k = 0; k < NC; k++) x[k] = lane < nw ? red[k][lane] : fe_zero();
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
#pragma unroll
      for (int k = 0; k < NC; k++) x[k] = fadd(x[k], shfl_down_fe(x[k], d));
  }
}

// MODE 0: message over the pairs of in (pairs = m / 2).
// MODE 1: fold in (length 4 * pairs) by *r into out and message of the folded vectors.
// MODE 2: fold only (pairs = outputs).
// scale (optional): vector 2 of pair entry e is multiplied by scale[e >> scale_log]
// as it is read (the parties' weights of the cubic form).
template <int FORM, int MODE>
__global__ void __launch_bounds__(kThreads) form_step_kernel(RoundArgs a) {
  constexpr int NV = Form<FORM>::NV, NC = Form<FORM>::NC;
  fe acc[NC];
#pragma unroll
  for (int k = 0; k < NC; k++) acc[k] = fe_zero();
  const fe r = MODE ? *a.r : fe_zero();
  const fe b = a.b ? *a.b : fe_zero();
  const uint64_t stride = (uint64_t)gridDim.x * kThreads;
  for (uint64_t g = (uint64_t)blockIdx.x * kThreads + threadIdx.x; g < a.pairs; g += stride) {
    Line l[NV];
    if (MODE == 0) {
#pragma unroll
      for (int k = 0; k < NV; k++) {
        fe lo = a.in[k][2 * g], hi = a.in[k][2 * g + 1];
        if (k == 2 && a.scale) {  // a pair may straddle two parties when M = 1
          lo = fmul(lo, a.scale[(2 * g) >> a.scale_log]);
          hi = fmul(hi, a.scale[(2 * g + 1) >> a.scale_log]);
        }
        l[k] = line(lo, hi);
      }
      accumulate<FORM>(l, b, acc);
    } else if (MODE == 1) {
      // every vector's four entries are loaded before any output is stored
      // (the stores could alias later loads, so the compiler would not
      // hoist them): one memory round trip per step instead of one per vector
      fe xs[NV][4];
#pragma unroll
      for (int k = 0; k < NV; k++) {
        const fe *p = a.in[k] + 4 * g;
#pragma unroll
        for (int q = 0; q < 4; q++) xs[k][q] = p[q];
      }
#pragma unroll
      for (int k = 0; k < NV; k++) {
        fe x0 = xs[k][0], x1 = xs[k][1], x2 = xs[k][2], x3 = xs[k][3];
        if (k == 2 && a.scale) {
          x0 = fmul(x0, a.scale[(4 * g) >> a.scale_log]);
          x1 = fmul(x1, a.scale[(4 * g + 1) >> a.scale_log]);
          x2 = fmul(x2, a.scale[(4 * g + 2) >> a.scale_log]);
          x3 = fmul(x3, a.scale[(4 * g + 3) >> a.scale_log]);
        }
        const fe f0 = fadd(x0, fmul(r, fsub(x1, x0)));
        const fe f1 = fadd(x2, fmul(r, fsub(x3, x2)));
        a.out[k][2 * g] = f0;
        a.out[k][2 * g + 1] = f1;
        l[k] = line(f0, f1);
      }
      accumulate<FORM>(l, b, acc);
    } else {
#pragma unroll
      for (int k = 0; k < NV; k++) {
        fe x0 = a.in[k][2 * g], x1 = a.in[k][2 * g + 1];
        if (k == 2 && a.scale) {
          x0 = fmul(x0, a.scale[(2 * g) >> a.scale_log]);
          x1 = fmul(x1, a.scale[(2 * g + 1) >> a.scale_log]);
        }
        a.out[k][g] = fadd(x0, fmul(r, fsub(x1, x0)));
      }
    }
  }
  if (MODE == 2) return;
  acc_to_coeffs<FORM>(acc);
  block_sum<NC>(acc);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NC; k++) a.partial[(uint64_t)blockIdx.x * NC + k] = acc[k];
}

// Copies the first entry of every vector (with the weight scale of vector
// 2) to fin: the final values when no round is left.
__global__ void form_first_kernel(RoundArgs a, int nv, fe *fin) {
  const int k = threadIdx.x;
  if (k >= nv) return;
  fe x = a.in[k][0];
  if (k == 2 && a.scale) x = fmul(x, a.scale[0]);
  fin[k] = x;
}

__device__ fe eval_poly(const fe *c, int nc, fe x) {
  fe acc = c[0];
  for (int k = 1; k < nc; k++) acc = fadd(fmul(acc, x), c[k]);
  return acc;
}

// Thread-0 part of a round: checks H(0) + H(1) against the running claim y,
// stores H, draws the challenge (Fiat-Shamir hash chain fs over the
// coefficients, or the leader's glibc challenge drawn ahead of time by
// prng_draw_kernel when drawn is set) and updates the claim.  The state is
// passed by reference so that the one-CTA tail keeps it in registers.
__device__ fe finish_round(const fe *H, int nc, fe &fs, fe &y, uint32_t &error, int round, const fe *drawn,
                           fe *polys, fe *chal) {
  // H(0) + H(1) = 2 c_last + sum of the other coefficients
  fe s = H[nc - 1];
  for (int k = 0; k < nc; k++) s = fadd(s, H[k]);
  if (!fe_eq(s, y)) error |= 1u;
  for (int k = 0; k < nc; k++) polys[(uint64_t)round * nc + k] = H[k];
  fe ch;
  if (drawn) {
    ch = *drawn;
  } else {
    for (int k = 0; k < nc; k++) fs = hash_F(fs, H[k]);
    ch = fs;
  }
  chal[round] = ch;
  y = eval_poly(H, nc, ch);
  return ch;
}

// Sums the partials into the round polynomial H (nc coefficients) and
// finishes the round.
__global__ void form_finalize_kernel(const fe *partial, int blocks, int nc, RoundState *st, int round,
                                     const fe *drawn, fe *polys, fe *chal) {
  __shared__ fe red[4][kThreads];
  fe acc[4] = {fe_zero(), fe_zero(), fe_zero(), fe_zero()};
  for (int i = threadIdx.x; i < blocks; i += kThreads)
    for (int k = 0; k < nc; k++) acc[k] = fadd(acc[k], partial[(uint64_t)i * nc + k]);
  for (int k = 0; k < 4; k++) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < 4; k++) red[k][threadIdx.x] = fadd(red[k][threadIdx.x], red[k][threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x) return;
  fe H[4];
  for (int k = 0; k < nc; k++) H[k] = red[k][0];
  fe fs = st->fs, y = st->y;
  uint32_t error = st->error;
  finish_round(H, nc, fs, y, error, round, drawn, polys, chal);
  st->fs = fs;
  st->y = y;
  st->error = error;
}

// The leader's rounds take the fourth of every four F::_random() draws
// (Distributed_Sumcheck.cpp); the glibc stream depends on nothing the rounds
// compute, so its n challenges are drawn in one thread while the first,
// largest rounds run, and the stream's final state goes back to st->prng.
__global__ void prng_draw_kernel(RoundState *st, int n, fe *out) {
  __shared__ glibc_prng g;  // dynamically indexed table: work on a shared copy
  if (threadIdx.x) return;
  g = st->prng;
  for (int j = 0; j < n; j++) {
    fe ch;
    for (int k = 0; k < 4; k++) ch = prng_field(g);
    out[j] = ch;
  }
  st->prng = g;
}

constexpr int kTailThreads = 512;

struct TailArgs {
  const fe *in[3];  // entries entering round i0, before its fold
  fe *buf[2][3];    // ping-pong outputs (buf[0] differs from in)
  uint64_t cur;     // entries of every vector entering round i0
  int i0, total, fs_rounds;
  RoundState *st;
  const fe *drawn;  // glibc challenges of rounds fs_rounds.. (or null)
  fe *polys, *chal, *fin;
};

// Rounds i0..total-1 of the party sumcheck and the final fold in one CTA,
// once the vectors are small: every round is the fused fold + message of
// form_step_kernel<FORM, 1>, a block reduction and finish_round, with no
// launch between rounds.
template <int FORM>
__global__ void __launch_bounds__(kTailThreads) form_tail_kernel(TailArgs t) {
  constexpr int NV = Form<FORM>::NV, NC = Form<FORM>::NC;
  __shared__ fe red[NC][kTailThreads / 32];
  __shared__ fe sh_r;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const fe *in[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) in[k] = t.in[k];
  fe r = t.chal[t.i0 - 1];
  fe fs = fe_zero(), y = fe_zero();  // the running state, in thread 0's registers
  uint32_t error = 0;
  if (threadIdx.x == 0) {
    fs = t.st->fs;
    y = t.st->y;
    error = t.st->error;
  }
  uint64_t cur = t.cur;
  int pp = 0;
  for (int i = t.i0; i < t.total; i++) {
    fe acc[NC];
#pragma unroll
    for (int k = 0; k < NC; k++) acc[k] = fe_zero();
    const uint64_t pairs = cur / 4;
    for (uint64_t g = threadIdx.x; g < pairs; g += kTailThreads) {
      fe xs[NV][4];
#pragma unroll
      for (int k = 0; k < NV; k++)
#pragma unroll
        for (int q = 0; q < 4; q++) xs[k][q] = in[k][4 * g + q];
      Line l[NV];
#pragma unroll
      for (int k = 0; k < NV; k++) {
        const fe f0 = fadd(xs[k][0], fmul(r, fsub(xs[k][1], xs[k][0])));
        const fe f1 = fadd(xs[k][2], fmul(r, fsub(xs[k][3], xs[k][2])));
        t.buf[pp][k][2 * g] = f0;
        t.buf[pp][k][2 * g + 1] = f1;
        l[k] = line(f0, f1);
      }
      accumulate<FORM>(l, fe_zero(), acc);
    }
    acc_to_coeffs<FORM>(acc);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
#pragma unroll
      for (int k = 0; k < NC; k++) acc[k] = fadd(acc[k], shfl_down_fe(acc[k], d));
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < NC; k++) red[k][wid] = acc[k];
    __syncthreads();  // also orders this round's stores before the next round's loads
    if (wid == 0) {
#pragma unroll
      for (int k = 0; k < NC; k++) acc[k] = red[k][lane % (kTailThreads / 32)];
      if (lane >= kTailThreads / 32)
#pragma unroll
        for (int k = 0; k < NC; k++) acc[k] = fe_zero();
#pragma unroll
      for (int d = 16; d > 0; d >>= 1)
#pragma unroll
        for (int k = 0; k < NC; k++) acc[k] = fadd(acc[k], shfl_down_fe(acc[k], d));
      if (lane == 0)
        sh_r = finish_round(acc, NC, fs, y, error, i,
                            i >= t.fs_rounds && t.drawn ? t.drawn + (i - t.fs_rounds) : nullptr, t.polys, t.chal);
    }
    __syncthreads();
    r = sh_r;
#pragma unroll
    for (int k = 0; k < NV; k++) in[k] = t.buf[pp][k];
    pp ^= 1;
    cur /= 2;
  }
  if (threadIdx.x == 0) {
    t.st->fs = fs;
    t.st->y = y;
    t.st->error = error;
  }
  // final fold of the last length-2 vectors: the leader's v[0] values
#pragma unroll
  for (int k = 0; k < NV; k++)
    if ((int)threadIdx.x == k) t.fin[k] = fadd(in[k][0], fmul(r, fsub(in[k][1], in[k][0])));
}

// Rounds i0..rounds-1 of a sumcheck whose challenges were drawn ahead
// (the leader's glibc sumchecks of delegate_protocol.cpp) and its final
// fold, in one CTA: every round the fused fold + message, a block
// reduction, then thread 0 checks H(0) + H(1) against the running claim
// (flag `bit` when it differs, none when bit is 0), stores H, takes the
// round's challenge and updates the claim.
template <int FORM>
__global__ void __launch_bounds__(kTailThreads) form_tail_drawn_kernel(DrawnTailArgs t) {
  constexpr int NV = Form<FORM>::NV, NC = Form<FORM>::NC;
  __shared__ fe red[NC][kTailThreads / 32];
  __shared__ fe sh_r;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const fe *in[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) in[k] = t.in[k];
  fe r = t.ch[t.i0 - 1];
  fe y = fe_zero();
  if (threadIdx.x == 0) y = *t.y;
  int pp = 0;
  for (int i = t.i0; i < t.rounds; i++) {
    fe acc[NC];
#pragma unroll
    for (int k = 0; k < NC; k++) acc[k] = fe_zero();
    const uint64_t pairs = t.n >> (i + 1);
    for (uint64_t g = threadIdx.x; g < pairs; g += kTailThreads) {
      Line l[NV];
#pragma unroll
      for (int k = 0; k < NV; k++) {
        const fe *p = in[k] + 4 * g;
        const fe f0 = fadd(p[0], fmul(r, fsub(p[1], p[0])));
        const fe f1 = fadd(p[2], fmul(r, fsub(p[3], p[2])));
        t.buf[pp][k][2 * g] = f0;
        t.buf[pp][k][2 * g + 1] = f1;
        l[k] = line(f0, f1);
      }
      accumulate<FORM>(l, fe_zero(), acc);
    }
    acc_to_coeffs<FORM>(acc);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
#pragma unroll
      for (int k = 0; k < NC; k++) acc[k] = fadd(acc[k], shfl_down_fe(acc[k], d));
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < NC; k++) red[k][wid] = acc[k];
    __syncthreads();  // also orders this round's stores before the next round's loads
    if (wid == 0) {
#pragma unroll
      for (int k = 0; k < NC; k++) acc[k] = lane < kTailThreads / 32 ? red[k][lane] : fe_zero();
#pragma unroll
      for (int d = 16; d > 0; d >>= 1)
#pragma unroll
        for (int k = 0; k < NC; k++) acc[k] = fadd(acc[k], shfl_down_fe(acc[k], d));
      if (lane == 0) {
        fe s = acc[NC - 1];
        for (int k = 0; k < NC; k++) s = fadd(s, acc[k]);
        if (t.bit && !fe_eq(s, y)) atomicOr(t.flags, t.bit);
        for (int k = 0; k < NC; k++) put_fe(t.tr, t.off_polys + 16ull * ((uint64_t)i * NC + k), acc[k]);
        const fe c = t.draw[t.first + (uint64_t)t.stride * i];
        t.ch[i] = c;
        y = eval_poly(acc, NC, c);
        sh_r = c;
      }
    }
    __syncthreads();
    r = sh_r;
#pragma unroll
    for (int k = 0; k < NV; k++) in[k] = t.buf[pp][k];
    pp ^= 1;
  }
  if (threadIdx.x == 0) *t.y = y;
  // the final fold of the length-2 vectors: their v[0]
  if ((int)threadIdx.x < NV) {
    const fe *p = in[threadIdx.x];
    const fe v = fadd(p[0], fmul(r, fsub(p[1], p[0])));
    t.fin[threadIdx.x] = v;
    put_fe(t.tr, t.off_fin + 16ull * threadIdx.x, v);
  }
}

__global__ void form_sum_kernel(const fe *partial, int blocks, int nc, fe *out) {
  __shared__ fe red[kMaxFormCoeffs][kThreads];
  fe acc[kMaxFormCoeffs];
  for (int k = 0; k < kMaxFormCoeffs; k++) acc[k] = fe_zero();
  for (int i = threadIdx.x; i < blocks; i += kThreads)
    for (int k = 0; k < nc; k++) acc[k] = fadd(acc[k], partial[(uint64_t)i * nc + k]);
  for (int k = 0; k < kMaxFormCoeffs; k++) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < kMaxFormCoeffs; k++) red[k][threadIdx.x] = fadd(red[k][threadIdx.x], red[k][threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x < (unsigned)nc) out[threadIdx.x] = red[threadIdx.x][0];
}

template <int FORM, int MODE>
void launch_step(const RoundArgs &a, int blocks, cudaStream_t s) {
  form_step_kernel<FORM, MODE><<<blocks, kThreads, 0, s>>>(a);
  GBZ_CUDA(cudaGetLastError());
}

template <int FORM>
void launch_form(const RoundArgs &a, int mode, int blocks, cudaStream_t s) {
  if (mode == 0) launch_step<FORM, 0>(a, blocks, s);
  else if (mode == 1) launch_step<FORM, 1>(a, blocks, s);
  else launch_step<FORM, 2>(a, blocks, s);
}

}  // namespace

int form_vectors(int form) {
  switch (form) {
    case SC_QUADRATIC: return 2;
    case SC_CUBIC: return 3;
    case SC_BATCH: return 6;
    case SC_ZEROCHECK: return 6;
    case SC_QUADRUPLE: return 4;
    default: return 0;
  }
}
int form_coeffs(int form) {
  switch (form) {
    case SC_QUADRATIC: return 3;
    case SC_CUBIC: return 4;
    case SC_BATCH: return 3;
    case SC_ZEROCHECK: return 4;
    case SC_QUADRUPLE: return 5;
    default: return 0;
  }
}

int round_blocks(uint64_t pairs) {
  uint64_t want = (pairs + kThreads - 1) / kThreads;
  const uint64_t cap = 152 * 8;
  if (want > cap) want = cap;
  return want ? (int)want : 1;
}

void form_step_launch(int form, const RoundArgs &a, int mode, int blocks, cudaStream_t s) {
  switch (form) {
    case SC_QUADRATIC: launch_form<SC_QUADRATIC>(a, mode, blocks, s); break;
    case SC_CUBIC: launch_form<SC_CUBIC>(a, mode, blocks, s); break;
    case SC_BATCH: launch_form<SC_BATCH>(a, mode, blocks, s); break;
    case SC_ZEROCHECK: launch_form<SC_ZEROCHECK>(a, mode, blocks, s); break;
    case SC_QUADRUPLE: launch_form<SC_QUADRUPLE>(a, mode, blocks, s); break;
    default: throw ArgError("sumcheck: unknown round form");
  }
}

void form_tail_drawn_launch(int form, const DrawnTailArgs &a, cudaStream_t s) {
  switch (form) {
    case SC_QUADRATIC: form_tail_drawn_kernel<SC_QUADRATIC><<<1, kTailThreads, 0, s>>>(a); break;
    case SC_CUBIC: form_tail_drawn_kernel<SC_CUBIC><<<1, kTailThreads, 0, s>>>(a); break;
    case SC_QUADRUPLE: form_tail_drawn_kernel<SC_QUADRUPLE><<<1, kTailThreads, 0, s>>>(a); break;
    default: throw ArgError("sumcheck tail: quadratic, cubic or quadruple form");
  }
  GBZ_CUDA(cudaGetLastError());
}

void form_sum_launch(const fe *partial, int blocks, int nc, fe *out, cudaStream_t s) {
  form_sum_kernel<<<1, kThreads, 0, s>>>(partial, blocks, nc, out);
  GBZ_CUDA(cudaGetLastError());
}

void form_finalize_launch(const fe *partial, int blocks, int nc, RoundState *st, int round, const fe *drawn, fe *polys,
                          fe *chal, cudaStream_t s) {
  form_finalize_kernel<<<1, kThreads, 0, s>>>(partial, blocks, nc, st, round, drawn, polys, chal);
  GBZ_CUDA(cudaGetLastError());
}

void form_first_launch(const RoundArgs &a, int nv, fe *fin, cudaStream_t s) {
  form_first_kernel<<<1, 32, 0, s>>>(a, nv, fin);
  GBZ_CUDA(cudaGetLastError());
}

int party_sumcheck_rounds(uint64_t M, int N, int offset, int *fs_rounds) {
  const int lm = ilog2(M);
  int rounds = lm - offset, off = offset;
  if (rounds <= 0) {
    rounds = 0;
    off = lm;
  }
  if (fs_rounds) *fs_rounds = rounds;
  return rounds + ilog2((uint64_t)N << off);
}

void party_sumcheck_enqueue(int form, const fe *const *v, uint64_t M, int N, const fe *w, int offset, RoundState *st,
                            fe *const *scratch, fe *partial, fe *polys, fe *chal, fe *fin, fe *drawn,
                            const SideStream &side, cudaStream_t s) {
  // The N parties' vectors are held party-major, so pair g of the
  // concatenation is pair g mod (cur/2) of party g / (cur/2) while every
  // party still has two entries or more: the parties' round polynomials
  // summed (with the weights w folded into v3 for the cubic form, which is
  // what aggregate_poly computes) are the round polynomial of the
  // concatenation, and the leader's gathered vectors are the concatenation
  // itself.  So the N-party prover is one sumcheck over N * M entries whose
  // first rounds draw Fiat-Shamir challenges and whose last log2(N * 2^offset)
  // rounds draw the leader's glibc challenges.
  const int nv = form_vectors(form), nc = form_coeffs(form);
  int fs_rounds = 0;
  const int total = party_sumcheck_rounds(M, N, offset, &fs_rounds);
  uint64_t cur = M * (uint64_t)N;
  RoundArgs a{};
  a.b = nullptr;
  a.partial = partial;
  a.scale = form == SC_CUBIC ? w : nullptr;
  a.scale_log = ilog2(M);
  for (int k = 0; k < nv; k++) a.in[k] = v[k];
  if (total == 0) {
    form_first_launch(a, nv, fin, s);
    return;
  }
  // the leader's glibc challenges, drawn on the side stream while the first
  // rounds run; the stream joins before the first round that takes one
  const bool glibc = total > fs_rounds;
  if (glibc) {
    cudaStream_t ds = side.stream ? side.stream : s;
    if (side.stream) {
      GBZ_CUDA(cudaEventRecord(side.fork, s));
      GBZ_CUDA(cudaStreamWaitEvent(side.stream, side.fork, 0));
    }
    prng_draw_kernel<<<1, 32, 0, ds>>>(st, total - fs_rounds, drawn);
    GBZ_CUDA(cudaGetLastError());
    if (side.stream) GBZ_CUDA(cudaEventRecord(side.join, side.stream));
  }
  bool joined = !glibc || !side.stream;
  auto join = [&](int upto) {  // before a launch that finishes rounds up to upto
    if (!joined && upto >= fs_rounds) {
      GBZ_CUDA(cudaStreamWaitEvent(s, side.join, 0));
      joined = true;
    }
  };
  int pp = 0;
  for (int i = 0; i < total; i++) {
    int blocks;
    if (i == 0) {
      a.pairs = cur / 2;
      blocks = round_blocks(a.pairs);
      form_step_launch(form, a, 0, blocks, s);
    } else {
      if (i >= 2 && cur <= kTailEntries) {
        // the remaining rounds and the final fold in one CTA
        TailArgs t{};
        for (int k = 0; k < nv; k++) {
          t.in[k] = a.in[k];
          t.buf[0][k] = scratch[pp * 6 + k];
          t.buf[1][k] = scratch[(pp ^ 1) * 6 + k];
        }
        t.cur = cur;
        t.i0 = i;
        t.total = total;
        t.fs_rounds = fs_rounds;
        t.st = st;
        t.drawn = glibc ? drawn : nullptr;
        t.polys = polys;
        t.chal = chal;
        t.fin = fin;
        join(total - 1);
        if (form == SC_QUADRATIC) form_tail_kernel<SC_QUADRATIC><<<1, kTailThreads, 0, s>>>(t);
        else form_tail_kernel<SC_CUBIC><<<1, kTailThreads, 0, s>>>(t);
        GBZ_CUDA(cudaGetLastError());
        return;
      }
      // fold by the previous challenge into scratch[pp], message of the result
      a.pairs = cur / 4;
      a.r = chal + (i - 1);
      for (int k = 0; k < nv; k++) a.out[k] = scratch[pp * 6 + k];
      blocks = round_blocks(a.pairs);
      form_step_launch(form, a, 1, blocks, s);
      for (int k = 0; k < nv; k++) a.in[k] = a.out[k];
      a.scale = nullptr;
      pp ^= 1;
      cur /= 2;
    }
    join(i);
    form_finalize_launch(partial, blocks, nc, st, i, i >= fs_rounds ? drawn + (i - fs_rounds) : nullptr, polys, chal,
                         s);
  }
  // final fold of the last length-2 vectors: the leader's v[0] values
  a.pairs = 1;
  a.r = chal + (total - 1);
  for (int k = 0; k < nv; k++) a.out[k] = fin + k;
  form_step_launch(form, a, 2, 1, s);
}

}  // namespace gbz
