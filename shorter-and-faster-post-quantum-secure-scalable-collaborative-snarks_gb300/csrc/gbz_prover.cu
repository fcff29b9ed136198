// The plain single-party prover on one GPU.
//
// One proof = the reference's call sequence
//   Whir_Commit_initial (Whir.cpp:158-190)          -> root
//   hash_to_field({0}) x log n (main.cpp:83-85)      -> evaluation point z
//   quadratic sumcheck of sum_x w(x) eq(z, x) with Fiat-Shamir challenges
//     (round body of _quadratic_cosumcheck, coSumcheck_MPI.cpp:195-219)
//   Whir_Open of the resulting claim, whir_k = 4 (Whir.cpp:388-467)
// and its transcript is the ordered record stream documented in
// include/gbz.h.  Everything, including the Fiat-Shamir chain and the glibc
// random() draws that the reference uses for WHIR challenges and queries,
// runs on the device: a proof is a fixed sequence of launches on one
// stream with no host synchronisation, so it can be replayed from a CUDA
// graph and overlapped with other proofs on other streams.
#include <math.h>

#include <cstring>
#include <memory>
#include <mutex>

#include "gbz_prover.cuh"

namespace gbz {

namespace {

// ------------------------------------------------------------ kernels


// The glibc generator state is worked on in shared memory by one thread and
// written back: its table is indexed dynamically, and hundreds of draws on
// the global copy would each pay a memory round trip.
__global__ void k_init(ProofState *st, uint32_t seed, int seed_in_state) {
  __shared__ glibc_prng g;
  st += blockIdx.x;  // a batch: one CTA per proof
  if (threadIdx.x) return;
  st->fs = fe_zero();
  prng_seed(g, seed_in_state ? st->seed_in : seed);
  st->prng = g;
  st->y = fe_zero();
  st->K = fe_zero();
  st->error = 0;
}

// The state of an opening alone: the caller's generator, point and claim.
__global__ void k_init_open(ProofState *st, glibc_prng g, const fe *point, int logn, fe K) {
  if (threadIdx.x == 0) {
    st->fs = fe_zero();
    st->prng = g;
    st->y = fe_zero();
    st->K = K;
    st->error = 0;
  }
  for (int i = threadIdx.x; i < logn; i += blockDim.x) st->chal[i] = point[i];
}

// z_i = hash_to_field({0}) for i < logn.
__global__ void k_point(ProofState *st, int logn, uint8_t *tr, uint64_t off, uint64_t trs) {
  st += blockIdx.x;
  tr += trs * blockIdx.x;
  if (threadIdx.x) return;
  fe s = st->fs;
  for (int i = 0; i < logn; i++) {
    s = hash_F(s, fe_zero());
    st->z[i] = s;
    put_fe(tr, off + 16 * i, s);
  }
  st->fs = s;
}

__device__ void sum_partials(const fe *partial, int blocks, fe out[3]) {
  __shared__ fe red[3][32];
  fe A = fe_zero(), C = fe_zero(), D = fe_zero();
  for (int i = threadIdx.x; i < blocks; i += blockDim.x) {
    A = fadd(A, partial[3 * i]);
    C = fadd(C, partial[3 * i + 1]);
    D = fadd(D, partial[3 * i + 2]);
  }
  for (int d = 16; d > 0; d >>= 1) {
    fe t;
    t.re = __shfl_down_sync(0xffffffffu, A.re, d); t.im = __shfl_down_sync(0xffffffffu, A.im, d); A = fadd(A, t);
    t.re = __shfl_down_sync(0xffffffffu, C.re, d); t.im = __shfl_down_sync(0xffffffffu, C.im, d); C = fadd(C, t);
    t.re = __shfl_down_sync(0xffffffffu, D.re, d); t.im = __shfl_down_sync(0xffffffffu, D.im, d); D = fadd(D, t);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { red[0][w] = A; red[1][w] = C; red[2][w] = D; }
  __syncthreads();
  if (threadIdx.x == 0) {
    A = C = D = fe_zero();
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      A = fadd(A, red[0][k]);
      C = fadd(C, red[1][k]);
      D = fadd(D, red[2][k]);
    }
    out[0] = A;
    out[1] = fsub(fsub(D, A), C);
    out[2] = C;
  }
}

// Round i of the sumcheck of sum w(x) eq(z, x) from the S(0), S(1) sums:
// H(X) = epre * eq1(z_i, X) * (S0 + X (S1 - S0)) (the reference's round
// message of the pairs of w and the folded eq vector); claim check; the
// Fiat-Shamir challenge hash_to_field({H.a, H.b, H.c}); y = H(c); and
// epre *= eq1(z_i, c).
__device__ fe sc_round_eq_apply(const fe SS[3], ProofState *st, int round, uint8_t *tr, int64_t off_claim,
                                uint64_t off_poly, uint64_t off_chal) {
  if (round == 0) st->epre = fe_one();
  const fe z = st->z[round], ep = st->epre;
  const fe a1 = fsub(fadd(z, z), fe_one()), b1 = fsub(fe_one(), z);
  const fe a2 = fsub(SS[2], SS[0]), b2 = SS[0];
  fe H[3];
  H[0] = fmul(ep, fmul(a1, a2));
  H[1] = fmul(ep, fadd(fmul(a1, b2), fmul(b1, a2)));
  H[2] = fmul(ep, fmul(b1, b2));
  fe h01 = fadd(quad_eval(H[0], H[1], H[2], fe_zero()), quad_eval(H[0], H[1], H[2], fe_one()));
  if (off_claim >= 0) {
    st->y = h01;
    put_fe(tr, (uint64_t)off_claim, h01);
  } else if (!fe_eq(h01, st->y)) {
    atomicOr(&st->error, 1u);
  }
  for (int k = 0; k < 3; k++) put_fe(tr, off_poly + 16 * k, H[k]);
  fe s = st->fs;
  for (int k = 0; k < 3; k++) s = hash_F(s, H[k]);
  st->fs = s;
  st->chal[round] = s;
  put_fe(tr, off_chal, s);
  st->y = quad_eval(H[0], H[1], H[2], s);
  st->epre = fmul(ep, fadd(b1, fmul(a1, s)));
  return s;
}

__global__ void k_sc_round_eq(const fe *partial, int blocks, ProofState *st, int round, uint8_t *tr,
                              int64_t off_claim, uint64_t off_poly, uint64_t off_chal, uint64_t ps, uint64_t trs) {
  partial = badv(partial, ps, blockIdx.x);
  st += blockIdx.x;
  tr += trs * blockIdx.x;
  fe SS[3];
  sum_partials(partial, blocks, SS);  // (S0, -S0-S1, S1)
  if (threadIdx.x) return;
  (void)sc_round_eq_apply(SS, st, round, tr, off_claim, off_poly, off_chal);
}

// The last rounds of the same sumcheck in one CTA, once w (m entries) and
// its eq table E (m / 2) fit in shared memory: per round r the fold of w by
// chal[r-1], the pairwise sums of E, the sums S(0), S(1) and the round
// itself (thread 0), with no launch or global round trip between rounds;
// then the final fold and the SC_FINAL record.  Round r's SC_POLY payload
// is at off_poly0 + 80 (r - round0), its SC_CHALLENGE 56 bytes after it.
constexpr int kScTailMax = 4096;
// Batched plans: codewords of 2^kBatchRealLog entries or more are committed
// proof by proof with the real-input transform, shorter ones in one batched
// general transform.
constexpr int kBatchRealLog = 18;
constexpr int kScTailThreads = 1024;
__global__ void __launch_bounds__(kScTailThreads)
k_sc_tail(ProofState *st, const fe *a, const fe *E, int m, int round0, int logn, uint8_t *tr, uint64_t off_poly0,
          uint64_t off_final, BStr bs) {
  extern __shared__ fe tail_sm[];
  // a batch: one CTA per proof; bs = strides of (a, E, tr)
  st += blockIdx.x;
  a = badv(a, bs.s[0], blockIdx.x);
  E = badv(E, bs.s[1], blockIdx.x);
  tr = badv(tr, bs.s[2], blockIdx.x);
  fe *w = tail_sm, *e = tail_sm + kScTailMax;
  __shared__ fe red[2][kScTailThreads / 32];
  __shared__ fe chal_s;
  for (int j = threadIdx.x; j < m; j += blockDim.x) w[j] = a[j];
  for (int j = threadIdx.x; j < m / 2; j += blockDim.x) e[j] = E[j];
  if (threadIdx.x == 0) chal_s = st->chal[round0 - 1];
  __syncthreads();
  for (int r = round0; r <= logn; r++) {
    // fold w by the previous challenge; E to pairwise sums (r < logn)
    const fe c = chal_s;
    const int half = m / 2;
    fe nw[kScTailMax / 2 / kScTailThreads], ne[kScTailMax / 4 / kScTailThreads + 1];
    int k = 0;
    for (int j = threadIdx.x; j < half; j += blockDim.x, k++)
      nw[k] = fadd(fmul(c, fsub(w[2 * j + 1], w[2 * j])), w[2 * j]);
    k = 0;
    if (r < logn)
      for (int j = threadIdx.x; j < half / 2; j += blockDim.x, k++) ne[k] = fadd(e[2 * j], e[2 * j + 1]);
    __syncthreads();
    k = 0;
    for (int j = threadIdx.x; j < half; j += blockDim.x, k++) w[j] = nw[k];
    k = 0;
    if (r < logn)
      for (int j = threadIdx.x; j < half / 2; j += blockDim.x, k++) e[j] = ne[k];
    m = half;
    __syncthreads();
    if (r == logn) break;
    // S(0) = sum w[2j] E[j], S(1) = sum w[2j+1] E[j]
    fe S0 = fe_zero(), S1 = fe_zero();
    for (int j = threadIdx.x; j < m / 2; j += blockDim.x) {
      S0 = fadd(S0, fmul(w[2 * j], e[j]));
      S1 = fadd(S1, fmul(w[2 * j + 1], e[j]));
    }
    for (int d = 16; d > 0; d >>= 1) {
      fe t;
      t.re = __shfl_down_sync(0xffffffffu, S0.re, d); t.im = __shfl_down_sync(0xffffffffu, S0.im, d); S0 = fadd(S0, t);
      t.re = __shfl_down_sync(0xffffffffu, S1.re, d); t.im = __shfl_down_sync(0xffffffffu, S1.im, d); S1 = fadd(S1, t);
    }
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = S0;
      red[1][threadIdx.x >> 5] = S1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      fe A = fe_zero(), B = fe_zero();
      for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
        A = fadd(A, red[0][q]);
        B = fadd(B, red[1][q]);
      }
      const fe SS[3] = {A, fe_zero(), B};
      const uint64_t op = off_poly0 + 80ull * (uint64_t)(r - round0);
      chal_s = sc_round_eq_apply(SS, st, r, tr, -1, op, op + 56);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {  // k_sc_final: the folded w and the eq prefix
    put_fe(tr, off_final, w[0]);
    put_fe(tr, off_final + 16, st->epre);
    st->K = w[0];
  }
}

__global__ void k_sc_final(ProofState *st, const fe *v1, const fe *v2, uint8_t *tr, uint64_t off, BStr bs) {
  st += blockIdx.x;
  v1 = badv(v1, bs.s[0], blockIdx.x);
  if (v2) v2 = badv(v2, bs.s[1], blockIdx.x);
  tr = badv(tr, bs.s[2], blockIdx.x);
  if (threadIdx.x) return;
  // v2 == nullptr: the eq vector was not folded, its last value is epre
  fe a = v1[0], b = v2 ? v2[0] : st->epre;
  put_fe(tr, off, a);
  put_fe(tr, off + 16, b);
  st->K = a;  // Whir_Open: K = claims[0].first
}


// omega^e from a two-level power table (lo[e & 4095] * hi[e >> 12]).
__device__ __forceinline__ fe pow_table(const fe *lo, const fe *hi, uint64_t e) {
  return fmul(lo[e & 4095u], hi[e >> 12]);
}

struct QueryArgs {
  ProofState *st;
  uint64_t cws, trs;     // per-proof strides of cw and tr in a batch (one CTA per proof)
  const fe *cw;          // previous codeword
  uint64_t L;            // its length
  uint64_t NL;           // new codeword length
  int l;                 // number of queries
  uint8_t *tr;
  uint64_t off_q, off_rep, off_ans, off_path, off_comb, off_K;
  // omega_L^{-e} and omega_NL^{e} tables, and per-iteration constants of
  // get_RS_multifold_segment_tensor for a segment of 4 (coPCS_utils.cpp:333-383)
  const fe *inv_lo, *inv_hi, *new_lo, *new_hi;
  fe step0;    // (omega_L^{-1})^(L/4): advance of inv_omegas at level 0
  fe len_inv;  // 4^{-1}
};


// The WHIR randomness of a proof, drawn up front.  Every F::_random() and
// rand() of the opening comes from the glibc generator seeded once, and no
// draw depends on the data, so the draws of Whir_Open in their order
// (per iteration: the two round challenges of whir_sumcheck, the l query
// positions of whir_query, update_betas' r; then the final point,
// Whir.cpp:233-249, 262-268, 327, 426-446) can be made before the
// opening starts.
struct SchedArgs {
  int T;                            // iterations
  int l[kMaxWhirIter];              // queries per iteration
  int32_t qmod[kMaxWhirIter];       // codeword length / 4 per iteration
  int lg_final;                     // log2 of the final polynomial's length
};
constexpr int kFieldDraws = 40;     // random() outputs behind one F::_random() (two 20-digit numbers)
constexpr int kMaxDraws = kMaxWhirIter * (3 * kFieldDraws + kMaxQueries) + 8 * kFieldDraws;

// randomNumber (fieldElement.cpp:363-368) from 20 consecutive outputs.
__device__ uint64_t number_from(const int32_t *d) {
  uint64_t ret = (uint64_t)(d[0] % 10);
  for (int i = 1; i < 20; i++) {
    ret = ret * 10ull + (uint64_t)(d[i] % 10);
    ret = ret >= P ? ret % P : ret;
  }
  return ret;
}

// One thread runs the generator with its 31-word table in registers (the
// table rotated so that the front index is 3 and the rear 0, which makes
// every index of a 31-draw cycle a constant) and stores the N outputs in
// shared memory; then all threads derive the field elements (40 outputs
// each) and the query positions from them.
__global__ void __launch_bounds__(256) k_whir_schedule(ProofState *st, SchedArgs a) {
  __shared__ int32_t draws[kMaxDraws];
  st += blockIdx.x;
  int N = kFieldDraws * a.lg_final;
  for (int t = 0; t < a.T; t++) N += 3 * kFieldDraws + a.l[t];
  if (threadIdx.x == 0) {
    const int f0 = st->prng.f;
    uint32_t reg[31];
#pragma unroll
    for (int k = 0; k < 31; k++) reg[k] = (uint32_t)st->prng.tbl[(k + f0 + 28) % 31];
    for (int n = 0; n < N; n += 31) {
#pragma unroll
      for (int j = 0; j < 31; j++) {
        if (n + j < N) {
          reg[(j + 3) % 31] += reg[j];
          draws[n + j] = (int32_t)(reg[(j + 3) % 31] >> 1);
        }
      }
    }
    // the table in place, both indices advanced by N (glibc's state after N draws)
#pragma unroll
    for (int k = 0; k < 31; k++) st->prng.tbl[(k + f0 + 28) % 31] = (int32_t)reg[k];
    const int f = (f0 + N) % 31;
    st->prng.f = f;
    st->prng.r = (f + 28) % 31;
  }
  __syncthreads();
  // per iteration: r0, r1 (40 outputs each), l queries, update_betas' r; then the final point
  int off = 0;
  for (int t = 0; t < a.T; t++) {
    const int l = a.l[t];
    for (int i = threadIdx.x; i < l; i += blockDim.x) st->wq[t][i] = draws[off + 2 * kFieldDraws + i] % a.qmod[t];
    if (threadIdx.x < 3) {
      const int o = threadIdx.x < 2 ? off + kFieldDraws * threadIdx.x : off + 2 * kFieldDraws + l;
      const fe v = fe_make(number_from(draws + o) % P, number_from(draws + o + 20) % P);
      if (threadIdx.x < 2) st->wr[t][threadIdx.x] = v;
      else st->wrb[t] = v;
    }
    off += 3 * kFieldDraws + l;
  }
  for (int i = threadIdx.x; i < a.lg_final; i += blockDim.x) {
    const int o = off + kFieldDraws * i;
    st->fin_r[i] = fe_make(number_from(draws + o) % P, number_from(draws + o + 20) % P);
  }
}

// Preparation of an iteration's update_betas by the round kernel: scaled
// queries 2 q_i, omega_NL^{2 q_i} and the weights c_i = r^(i+1).
struct UbPrep {
  int l;                 // 0: no preparation
  const fe *lo, *hi;     // omega_NL^e
};
// The two WHIR sumcheck rounds of iteration t from the partials of the fused
// two-round pass, in one launch: each message is recorded (transcript and
// st->whw for the query chain, which checks it against K) with its challenge
// drawn up front, and the threads prepare the iteration's update_betas.
__global__ void k_whir_rounds2_s(const fe *partial0, const fe *partial1, int blocks, ProofState *st, int t,
                                 uint8_t *tr, uint64_t off_poly0, uint64_t off_chal0, uint64_t off_poly1,
                                 uint64_t off_chal1, UbPrep u, uint64_t ps, uint64_t trs) {
  partial0 = badv(partial0, ps, blockIdx.x);
  partial1 = badv(partial1, ps, blockIdx.x);
  st += blockIdx.x;
  tr += trs * blockIdx.x;
  fe H0[3], H1[3];
  sum_partials(partial0, blocks, H0);
  __syncthreads();  // sum_partials' shared scratch is reused
  sum_partials(partial1, blocks, H1);
  for (int j = threadIdx.x; j < u.l; j += blockDim.x) {
    const uint32_t q2 = 2u * (uint32_t)st->wq[t][j];
    st->q[j] = (int32_t)q2;
    st->omega_q[j] = pow_table(u.lo, u.hi, q2);
    st->comb[j] = fpow(st->wrb[t], (uint64_t)j + 1);
  }
  if (threadIdx.x) return;
  for (int k = 0; k < 3; k++) {
    put_fe(tr, off_poly0 + 16 * k, H0[k]);
    st->whw[t][0][k] = H0[k];
    put_fe(tr, off_poly1 + 16 * k, H1[k]);
    st->whw[t][1][k] = H1[k];
  }
  put_fe(tr, off_chal0, st->wr[t][0]);
  put_fe(tr, off_chal1, st->wr[t][1]);
}

// whir_query (Whir.cpp:251-314) of iteration t with the drawn positions, and
// the running claim of whir_sumcheck and update_betas: K is checked against
// both round messages (K == h(0) + h(1), K = h(r)), then K += sum_i c_i y_i
// (Whir.cpp:383-384).  Thread i handles query i.
__global__ void __launch_bounds__(kMaxQueries) k_whir_query_s(QueryArgs a, int t) {
  __shared__ fe red[kMaxQueries / 32];
  a.st += blockIdx.x;
  a.cw = badv(a.cw, a.cws, blockIdx.x);
  a.tr += a.trs * blockIdx.x;
  ProofState *st = a.st;
  const int i = threadIdx.x;
  fe contrib = fe_zero();
  if (i < a.l) {
    const int32_t q = st->wq[t][i];
    const uint64_t qi = (uint64_t)q;
    reinterpret_cast<int32_t *>(a.tr + a.off_q)[i] = q;
    fe seg[kWhirK];
    for (int j = 0; j < kWhirK; j++) {
      seg[j] = a.cw[qi + j * (a.L / kWhirK)];
      put_fe(a.tr, a.off_rep + 16 * (kWhirK * i + j), seg[j]);
    }
    // get_RS_multifold_segment_tensor(seg, r, L, qi) with r = the two WHIR
    // round challenges: level 0 pairs (j, j+2) with omega_L^{-(qi + j L/4)},
    // level 1 pairs (0, 1) with omega_{L/2}^{-qi} = omega_L^{-2 qi}.
    const fe one = fe_one(), r0 = st->wr[t][0], r1 = st->wr[t][1];
    fe inv_om = pow_table(a.inv_lo, a.inv_hi, qi);
    fe part[2];
    for (int j = 0; j < 2; j++) {
      fe s = fadd(seg[j], seg[j + 2]), d = fsub(seg[j], seg[j + 2]);
      part[j] = fadd(fmul(fsub(one, r0), s), fmul(fmul(r0, inv_om), d));
      inv_om = fmul(inv_om, a.step0);
    }
    fe po = pow_table(a.inv_lo, a.inv_hi, (2 * qi) & (a.L - 1));
    fe s = fadd(part[0], part[1]), d = fsub(part[0], part[1]);
    fe y = fmul(a.len_inv, fadd(fmul(fsub(one, r1), s), fmul(r1, fmul(po, d))));
    put_fe(a.tr, a.off_ans + 16 * i, y);
    const fe c = fpow(st->wrb[t], (uint64_t)i + 1);
    put_fe(a.tr, a.off_comb + 16 * i, c);
    contrib = fmul(c, y);
  }
  for (int dd = 16; dd > 0; dd >>= 1) {
    fe v;
    v.re = __shfl_down_sync(0xffffffffu, contrib.re, dd);
    v.im = __shfl_down_sync(0xffffffffu, contrib.im, dd);
    contrib = fadd(contrib, v);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = contrib;
  __syncthreads();
  if (threadIdx.x == 0) {
    fe K = st->K;
    for (int r = 0; r < kWhirLogK; r++) {
      const fe *h = st->whw[t][r];
      const fe h01 = fadd(quad_eval(h[0], h[1], h[2], fe_zero()), quad_eval(h[0], h[1], h[2], fe_one()));
      if (!fe_eq(h01, K)) atomicOr(&st->error, 2u);
      K = quad_eval(h[0], h[1], h[2], st->wr[t][r]);
    }
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) K = fadd(K, red[w]);
    st->K = K;
    put_fe(a.tr, a.off_K, K);
  }
}

}  // namespace

// --------------------------------------- kernels shared with the batch opening

// WHIR sumcheck round (whir_sumcheck, Whir.cpp:233-249): message h, the
// consistency check K == h(0) + h(1), challenge F::_random(), K = h(r).
__global__ void k_whir_round(const fe *partial, int blocks, ProofState *st, int i, uint8_t *tr,
                             uint64_t off_poly, uint64_t off_chal) {
  fe H[3];
  sum_partials(partial, blocks, H);
  if (threadIdx.x) return;
  fe h01 = fadd(quad_eval(H[0], H[1], H[2], fe_zero()), quad_eval(H[0], H[1], H[2], fe_one()));
  if (!fe_eq(h01, st->K)) atomicOr(&st->error, 2u);
  for (int k = 0; k < 3; k++) {
    put_fe(tr, off_poly + 16 * k, H[k]);
    st->hw[i][k] = H[k];
  }
  __shared__ glibc_prng g;
  g = st->prng;
  fe r = prng_field(g);
  st->prng = g;
  st->rw[i] = r;
  put_fe(tr, off_chal, r);
  st->K = quad_eval(H[0], H[1], H[2], r);
}

// ---- the Merkle nodes a proof reveals ------------------------------------
// create_tree_blake (merkle_tree.cpp:267-299) hashes the LEFT child twice,
// so node i of level k is G^k(leaf i 2^k) with G(h) = blake3(h || h), and
// leaf j = blake3(e[4j..4j+3]) (MT_commit_Blake, merkle_tree.cpp:195-233).
// The root and the authentication paths (open_tree_blake,
// merkle_tree.cpp:320-335) are therefore chains of compressions from single
// leaves; the prover computes only those instead of whole trees.  The same
// bytes as the full tree (gbz_merkle_commit_blake), which the transcript
// tests compare with the reference's.
__device__ __forceinline__ void leaf_hash(const fe *cw, uint64_t j, uint32_t h[8]) {
  uint32_t m[16];
  const uint4 *src = reinterpret_cast<const uint4 *>(cw + 4 * j);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const uint4 v = src[k];
    m[4 * k] = v.x; m[4 * k + 1] = v.y; m[4 * k + 2] = v.z; m[4 * k + 3] = v.w;
  }
  blake3_block64(m, h);
}
__device__ __forceinline__ void node_hash(uint32_t h[8]) {  // h <- blake3(h || h)
  uint32_t m[16];
#pragma unroll
  for (int k = 0; k < 8; k++) m[k] = m[8 + k] = h[k];
  blake3_block64(m, h);
}
__device__ __forceinline__ void put_hash(uint8_t *dst, const uint32_t h[8]) {  // 4-byte aligned
  uint32_t *d = reinterpret_cast<uint32_t *>(dst);
#pragma unroll
  for (int k = 0; k < 8; k++) d[k] = h[k];
}

// Root of the tree over a codeword of 4 * 2^depth elements: G^depth(leaf 0).
__device__ void merkle_root_dev(const fe *cw, int depth, uint8_t *tr, uint64_t off) {
  uint32_t h[8];
  leaf_hash(cw, 0, h);
  for (int d = 0; d < depth; d++) node_hash(h);
  put_hash(tr + off, h);
}
__global__ void k_merkle_root(const fe *cw, int depth, uint8_t *tr, uint64_t off) {
  if (threadIdx.x) return;
  merkle_root_dev(cw, depth, tr, off);
}
// The same for a batch: proof p (grid.x) reads cw + p cws, writes tr + p trs.
__global__ void k_merkle_root_b(const fe *cw, uint64_t cws, int depth, uint8_t *tr, uint64_t trs, uint64_t off) {
  if (threadIdx.x) return;
  merkle_root_dev(badv(cw, cws, blockIdx.x), depth, tr + trs * blockIdx.x, off);
}

// Authentication paths of the l queries: entry d of query i is the sibling
// (q >> d) ^ 1 of level d, i.e. G^d(leaf ((q >> d) ^ 1) << d).  One thread
// per entry, the deepest entries first.
__global__ void k_whir_paths_chain(const fe *cw, uint64_t leaves, int l, uint8_t *tr, uint64_t off_q,
                                   uint64_t off_path, uint64_t cws, uint64_t trs) {
  cw = badv(cw, cws, blockIdx.y);  // a batch: grid.y = proof
  tr += trs * blockIdx.y;
  const int depth = 63 - __clzll((long long)leaves);
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint64_t)l * depth) return;
  const int d = depth - 1 - (int)(t / l), i = (int)(t % l);
  const uint64_t q = (uint64_t)(uint32_t)reinterpret_cast<const int32_t *>(tr + off_q)[i];
  uint32_t h[8];
  leaf_hash(cw, ((q >> d) ^ 1ull) << d, h);
  for (int k = 0; k < d; k++) node_hash(h);
  put_hash(tr + off_path + 32ull * ((uint64_t)depth * i + d), h);
}

// The tree aggregate_commitments builds (Whir.cpp:594-605) has all-zero
// leaf hashes, so its level-d nodes all equal G^d(0): the root of a tree of
// 2^depth leaves, and every query's path entry d.
__global__ void k_zero_tree_root(int depth, uint8_t *tr, uint64_t off) {
  if (threadIdx.x) return;
  uint32_t h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int d = 0; d < depth; d++) node_hash(h);
  put_hash(tr + off, h);
}
__global__ void k_zero_tree_paths(int depth, int l, uint8_t *tr, uint64_t off_path) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;  // one thread per level
  if (d >= depth) return;
  uint32_t h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < d; k++) node_hash(h);
  for (int i = 0; i < l; i++) put_hash(tr + off_path + 32ull * ((uint64_t)depth * i + d), h);
}

// open_tree_blake (merkle_tree.cpp:320-335) for every query in a tree of
// `leaves` leaf hashes: sibling (pos >> d) ^ 1 of level d (levels stored back
// to back, level d starting at 2 leaves - 2 (leaves >> d)), one hash per
// thread so that all the scattered tree reads are in flight together.
__global__ void k_whir_paths(const uint8_t *tree, uint64_t leaves, int l, uint8_t *tr, uint64_t off_q,
                             uint64_t off_path) {
  const int depth = 63 - __clzll((long long)leaves);
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint64_t)l * depth) return;
  const int i = (int)(t / depth), d = (int)(t % depth);
  const uint64_t q = (uint64_t)(uint32_t)reinterpret_cast<const int32_t *>(tr + off_q)[i];
  const uint64_t lvl = 2 * leaves - 2 * (leaves >> d);
  const uint4 *src = reinterpret_cast<const uint4 *>(tree + 32 * (lvl + ((q >> d) ^ 1ull)));
  const uint4 h0 = src[0], h1 = src[1];
  // transcript payloads are only 4-byte aligned
  uint32_t *dst = reinterpret_cast<uint32_t *>(tr + off_path + 32ull * ((uint64_t)depth * i + d));
  dst[0] = h0.x; dst[1] = h0.y; dst[2] = h0.z; dst[3] = h0.w;
  dst[4] = h1.x; dst[5] = h1.y; dst[6] = h1.z; dst[7] = h1.w;
}

// Final round of Whir_Open (Whir.cpp:426-446) and of Whir_Batch_Open
// (:840-869): the remaining polynomial (m <= kFinalMax entries), log2 m
// F::_random draws and evaluate_vector(b, r).  With check_K, the flag 8 is
// raised unless K equals sum arr * b (verification step 2, :848-855).
__device__ void final_dev(ProofState *st, const fe *arr, const fe *b, int m, uint8_t *tr, uint64_t off_poly,
                          uint64_t off_point, uint64_t off_eval, int check_K, const fe *point, glibc_prng &g) {
  if (m < 1 || m > kFinalMax) {
    atomicOr(&st->error, 16u);
    return;
  }
  fe Kc = st->K;
  for (int i = 0; i < m; i++) {
    put_fe(tr, off_poly + 16 * i, arr[i]);
    Kc = fsub(Kc, fmul(arr[i], b[i]));
  }
  if (check_K && !fe_eq(Kc, fe_zero())) atomicOr(&st->error, 8u);
  const int lg = 31 - __clz(m);
  fe r[8];
  if (!point) g = st->prng;
  for (int i = 0; i < lg; i++) {
    r[i] = point ? point[i] : prng_field(g);
    put_fe(tr, off_point + 16 * i, r[i]);
  }
  if (!point) st->prng = g;
  fe v[kFinalMax];
  for (int i = 0; i < m; i++) v[i] = b[i];
  for (int i = 0; i < lg; i++) {
    fe om = fsub(fe_one(), r[i]);
    int L = 1 << (lg - 1 - i);
    for (int j = 0; j < L; j++) v[j] = fadd(fmul(om, v[2 * j]), fmul(r[i], v[2 * j + 1]));
  }
  put_fe(tr, off_eval, v[0]);
}
__global__ void k_final(ProofState *st, const fe *arr, const fe *b, int m, uint8_t *tr, uint64_t off_poly,
                        uint64_t off_point, uint64_t off_eval, int check_K, const fe *point) {
  __shared__ glibc_prng g;
  if (threadIdx.x) return;
  final_dev(st, arr, b, m, tr, off_poly, off_point, off_eval, check_K, point, g);
}
// The same for a batch of proofs whose final point was drawn up front
// (st->fin_r): proof p = grid.x, bs = strides of (arr, b, tr).
__global__ void k_final_b(ProofState *st, const fe *arr, const fe *b, int m, uint8_t *tr, uint64_t off_poly,
                          uint64_t off_point, uint64_t off_eval, BStr bs) {
  __shared__ glibc_prng g;
  if (threadIdx.x) return;
  st += blockIdx.x;
  final_dev(st, badv(arr, bs.s[0], blockIdx.x), badv(b, bs.s[1], blockIdx.x), m, badv(tr, bs.s[2], blockIdx.x),
            off_poly, off_point, off_eval, 0, st->fin_r, g);
}

// ------------------------------------------------------------ host side

bool update_betas_by_transform(int l, uint64_t nb, uint64_t N) {
  return ilog2(N) > 13 && ilog2(N) <= kMaxNttLogN && nb <= N && (uint64_t)l * nb > 4 * N;
}

int whir_query_count(int rate) { return (int)(-100.0 / log2(sqrt(1.0 / (double)rate))); }

uint64_t Layout::rec(uint32_t tag, uint32_t count, uint32_t unit) {
  uint64_t off = len;
  if (record_headers) {
    headers.push_back({off, tag, count});
  }
  len += 8 + (uint64_t)count * unit;
  return off + 8;
}

ProofPlan::~ProofPlan() {
  if (s2) cudaStreamSynchronize(s2);
  if (s3) cudaStreamSynchronize(s3);
  for (auto &g : graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
  }
  for (auto &kv : ntt) ntt_tables_free(kv.second);
  for (void *p : allocs) cudaFree(p);
  if (ev_in) cudaEventDestroy(ev_in);
  for (auto &e : ev_fold)
    if (e) cudaEventDestroy(e);
  for (auto &e : ev_commit)
    if (e) cudaEventDestroy(e);
  for (auto &e : ev_query)
    if (e) cudaEventDestroy(e);
  if (ev_sched) cudaEventDestroy(ev_sched);
  if (ev_root_tail) cudaEventDestroy(ev_root_tail);
  if (ev_init) cudaEventDestroy(ev_init);
  if (s2) cudaStreamDestroy(s2);
  if (s3) cudaStreamDestroy(s3);
}

void *ProofPlan::dalloc(uint64_t bytes) {
  void *p = nullptr;
  GBZ_CUDA(cudaMalloc(&p, bytes ? bytes : 16));
  allocs.push_back(p);
  return p;
}

NttTables &ProofPlan::tables(int lg) {
  auto it = ntt.find(lg);
  if (it != ntt.end()) return it->second;
  NttTables t;
  ntt_tables_build(t, lg);
  return ntt.emplace(lg, t).first->second;
}

std::unique_ptr<ProofPlan> plan_create(int logn, int rate, int batch) {
  if (logn < 3 || logn > 25) throw ArgError("prover: log2 witness length must be in [3, 25]");
  if (rate < 2 || rate > 64 || !is_pow2((uint64_t)rate)) throw ArgError("prover: rate must be a power of two in [2, 64]");
  if (batch < 1 || batch > 65535) throw ArgError("prover: 1..65535 proofs per plan");
  const uint64_t n = 1ull << logn, L = n * (uint64_t)rate;
  if (ilog2(L) > kMaxNttLogN) throw ArgError("prover: codeword longer than 2^26");
  auto p = std::unique_ptr<ProofPlan>(new ProofPlan());
  p->logn = logn;
  p->rate = rate;
  p->n = n;
  p->L = L;
  p->B = batch;
  const uint64_t B = (uint64_t)batch;
  p->bs_w = sizeof(fe) * n;
  p->bs_cw0 = sizeof(fe) * L;
  p->bs_cw1 = sizeof(fe) * (L / 2);
  p->bs_tmp = sizeof(fe) * L;
  p->bs_tmp2 = sizeof(fe) * (L / 2);
  p->bs_v = sizeof(fe) * (n / 2);
  p->bs_arr = sizeof(fe) * (n / 2);
  p->bs_beta = sizeof(fe) * n;
  p->bs_part = sizeof(fe) * 3 * (uint64_t)sc_blocks(n / 2);
  p->bs_ub = sizeof(fe) * kUpdateBetasScratch;
  p->w = (fe *)p->dalloc(B * p->bs_w);
  p->cw[0] = (fe *)p->dalloc(B * p->bs_cw0);
  p->cw[1] = (fe *)p->dalloc(B * p->bs_cw1);
  p->tmp = (fe *)p->dalloc(B * p->bs_tmp);
  p->tmp2 = (fe *)p->dalloc(B * p->bs_tmp2);
  GBZ_CUDA(cudaStreamCreateWithFlags(&p->s2, cudaStreamNonBlocking));
  GBZ_CUDA(cudaStreamCreateWithFlags(&p->s3, cudaStreamNonBlocking));
  GBZ_CUDA(cudaEventCreateWithFlags(&p->ev_in, cudaEventDisableTiming));
  GBZ_CUDA(cudaEventCreateWithFlags(&p->ev_sched, cudaEventDisableTiming));
  GBZ_CUDA(cudaEventCreateWithFlags(&p->ev_init, cudaEventDisableTiming));
  GBZ_CUDA(cudaEventCreateWithFlags(&p->ev_root_tail, cudaEventDisableTiming));
  for (auto &e : p->ev_fold) GBZ_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (auto &e : p->ev_commit) GBZ_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (auto &e : p->ev_query) GBZ_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  p->va[0] = (fe *)p->dalloc(B * p->bs_v);
  p->va[1] = (fe *)p->dalloc(B * p->bs_v);
  p->arr = (fe *)p->dalloc(B * p->bs_arr);
  p->vb[0] = (fe *)p->dalloc(B * p->bs_v);
  p->vb[1] = (fe *)p->dalloc(B * p->bs_v);
  p->beta = (fe *)p->dalloc(B * p->bs_beta);
  p->partial = (fe *)p->dalloc(B * p->bs_part);
  p->partial2 = (fe *)p->dalloc(B * p->bs_part);
  p->ub_scratch = (fe *)p->dalloc(B * p->bs_ub);
  p->st = (ProofState *)p->dalloc(B * sizeof(ProofState));
  GBZ_CUDA(cudaFuncSetAttribute(k_sc_tail, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(fe) * (kScTailMax + kScTailMax / 2))));
  // Build the transcript layout (record headers are constant).
  p->layout.record_headers = true;
  enqueue_proof(*p, nullptr, 1, nullptr, /*dry=*/true);  // layout and launch counts
  p->layout.record_headers = false;
  p->transcript_bytes = p->layout.len;
  p->transcript = (uint8_t *)p->dalloc(B * p->transcript_bytes);
  std::vector<uint8_t> img(p->transcript_bytes, 0);
  for (auto &h : p->layout.headers) {
    std::memcpy(&img[h.off], &h.tag, 4);
    std::memcpy(&img[h.off + 4], &h.count, 4);
  }
  for (uint64_t b = 0; b < B; b++)
    GBZ_CUDA(cudaMemcpy(p->transcript + b * p->transcript_bytes, img.data(), img.size(), cudaMemcpyHostToDevice));
  // Twiddle tables for every transform length the proof uses.
  p->tables(ilog2(L));
  for (uint64_t m = n, cur = (uint64_t)rate; m > 4; m /= 4, cur *= 2) {
    p->tables(ilog2(2 * cur * (m / 4)));
    p->tables(ilog2(cur * (m / 4)));  // the half-length update_betas transform
  }
  return p;
}

void plan_prepare_open(ProofPlan &p) {
  if (p.open_transcript) return;
  Layout saved = p.layout;
  const int launches = p.launches;
  int cat[PC_COUNT];
  for (int c = 0; c < PC_COUNT; c++) cat[c] = p.cat_launches[c];
  p.layout = Layout();
  p.layout.record_headers = true;
  OpenOnly o{};
  enqueue_proof(p, nullptr, 0, nullptr, /*dry=*/true, false, &o);
  const Layout open_layout = p.layout;
  p.layout = saved;
  p.launches = launches;
  for (int c = 0; c < PC_COUNT; c++) p.cat_launches[c] = cat[c];
  p.open_transcript_bytes = open_layout.len;
  p.open_transcript = (uint8_t *)p.dalloc(open_layout.len);
  std::vector<uint8_t> img(open_layout.len, 0);
  for (auto &h : open_layout.headers) {
    std::memcpy(&img[h.off], &h.tag, 4);
    std::memcpy(&img[h.off + 4], &h.count, 4);
  }
  GBZ_CUDA(cudaMemcpy(p.open_transcript, img.data(), img.size(), cudaMemcpyHostToDevice));
}

// Enqueue one proof.  witness: device pointer (nullptr: use plan->w).
// The dry run (dry = true) launches nothing; it fixes the transcript layout
// and counts the launches per category.
void enqueue_proof(ProofPlan &p, const fe *witness, uint32_t prng_seed, cudaStream_t s, bool dry, bool seed_in_state,
                   const OpenOnly *open) {
  Layout &lay = p.layout;
  lay.len = 0;
  if (dry) {
    p.launches = 0;
    for (int c = 0; c < PC_COUNT; c++) p.cat_launches[c] = 0;
  }
  const fe *w = witness ? witness : p.w;
  const int logn = p.logn;
  uint8_t *tr = open ? p.open_transcript : p.transcript;
  ProofState *st = p.st;
  // a batch: every launch covers the plan's B proofs (per-proof strides below)
  const int B = p.B;
  if (B > 1 && (open || (witness && witness != p.w))) throw ArgError("prover: a batch reads its witnesses from the plan");
  const uint64_t trs = p.transcript_bytes, sts = sizeof(ProofState);
  const uint64_t cw_s[2] = {p.bs_cw0, p.bs_cw1};
  Profiler *prof = (!dry && p.prof && p.prof->enabled) ? p.prof : nullptr;
  // RUN(category, kernel launches, statement): counts in the dry run, else
  // runs the statement (bracketed by profiler events when enabled).
#define RUN_ON(strm, cat, nlaunch, ...)        \
  do {                                         \
    if (dry) {                                 \
      p.launches += (nlaunch);                 \
      p.cat_launches[cat] += (nlaunch);        \
    } else {                                   \
      if (prof) prof->begin(cat, strm);        \
      __VA_ARGS__;                             \
      GBZ_CUDA(cudaGetLastError());            \
      if (prof) prof->end(strm);               \
    }                                          \
  } while (0)
#define RUN(cat, nlaunch, ...) RUN_ON(s, cat, nlaunch, __VA_ARGS__)

  // Commits go to the plan's second stream c; it starts after everything
  // the caller enqueued on s (the witness copy) and s joins it at the end.
  // With the profiler on, the commits stay on s so that the per-category
  // event times do not include waits for the other stream's kernels.
  cudaStream_t c = prof ? s : p.s2, q = prof ? s : p.s3;
  if (!dry) {
    GBZ_CUDA(cudaEventRecord(p.ev_in, s));
    GBZ_CUDA(cudaStreamWaitEvent(c, p.ev_in, 0));
  }
  if (open) {
    RUN(PC_PROTOCOL, 1, k_init_open<<<1, 32, 0, s>>>(st, open->prng, open->point, logn, open->K));
  } else {
    RUN(PC_PROTOCOL, 1, k_init<<<B, 32, 0, s>>>(st, prng_seed, seed_in_state ? 1 : 0));
  }
  // The opening's randomness, drawn on the query stream while the
  // commitment and the sumcheck run.
  {
    SchedArgs sa{};
    uint64_t mm = p.n, LL = p.L, cc = (uint64_t)p.rate;
    for (;;) {
      if (sa.T >= kMaxWhirIter) throw ArgError("prover: too many WHIR iterations");
      mm /= 4;
      sa.l[sa.T] = whir_query_count((int)cc);
      sa.qmod[sa.T] = (int32_t)(LL / 4);
      if (sa.l[sa.T] < 1 || sa.l[sa.T] > kMaxQueries) throw ArgError("prover: query count out of range");
      sa.T++;
      LL = 2 * cc * mm;
      cc *= 2;
      if (mm <= (uint64_t)kWhirK) break;
    }
    sa.lg_final = ilog2(mm);
    if (!dry) {
      GBZ_CUDA(cudaEventRecord(p.ev_init, s));
      GBZ_CUDA(cudaStreamWaitEvent(q, p.ev_init, 0));
    }
    RUN_ON(q, PC_PROTOCOL, 1, k_whir_schedule<<<B, 256, 0, q>>>(st, sa));
    if (!dry) GBZ_CUDA(cudaEventRecord(p.ev_sched, q));
  }

  // 1. commitment: codeword = NTT(w padded to rate*n), Merkle tree.
  uint64_t L = p.L;
  int cwi = 0;
  uint64_t off = lay.rec(T_COMMIT_ROOT, 1, 32);
  // The witness is expected in the base field (the imaginary words zero):
  // its transform is then a half-length transform of packed pairs
  // (ntt_launch_real); any other witness takes the general transform.
  if (open) {
    if (!dry && open->codeword != p.cw[0])
      GBZ_CUDA(cudaMemcpyAsync(p.cw[0], open->codeword, 16 * L, cudaMemcpyDeviceToDevice, c));
  } else if (B > 1 && ilog2(L) < kBatchRealLog) {
    // short codewords (launch bound): the batch's codewords as one batched
    // transform (the same values as the real-input path of a single proof)
    RUN_ON(c, PC_NTT, ntt_launch_count(ilog2(L)),
           ntt_launch_rows(p.tables(ilog2(L)), w, p.n, p.bs_w / sizeof(fe), p.cw[0], p.bs_cw0 / sizeof(fe), B, p.tmp,
                           false, c));
  } else if (B > 1) {
    // long codewords (integer-pipe bound): the real-input transform of each
    // proof, half the multiplies of the general one
    for (int pb = 0; pb < B; pb++) {
      if (!dry) GBZ_CUDA(cudaMemsetAsync(&st[pb].nonreal, 0, sizeof(uint32_t), c));
      RUN_ON(c, PC_NTT, ntt_launch_real_count(ilog2(L)),
             ntt_launch_real(p.tables(ilog2(L) - 1), p.tables(ilog2(L)),
                             reinterpret_cast<const fe *>(reinterpret_cast<const char *>(w) + p.bs_w * pb), p.n,
                             reinterpret_cast<fe *>(reinterpret_cast<char *>(p.cw[0]) + p.bs_cw0 * pb),
                             reinterpret_cast<fe *>(reinterpret_cast<char *>(p.tmp) + p.bs_tmp * pb), &st[pb].nonreal,
                             c));
    }
  } else {
    if (!dry) GBZ_CUDA(cudaMemsetAsync(&st->nonreal, 0, sizeof(uint32_t), c));
    RUN_ON(c, PC_NTT, ntt_launch_real_count(ilog2(L)),
           ntt_launch_real(p.tables(ilog2(L) - 1), p.tables(ilog2(L)), w, p.n, p.cw[0], p.tmp, &st->nonreal, c));
  }
  // The root (a chain of compressions from leaf 0) is computed on the query
  // stream once the codeword exists, off the chain of commits.
  uint64_t off_root[kMaxWhirIter + 1];
  off_root[0] = off;
  if (!dry) GBZ_CUDA(cudaEventRecord(p.ev_commit[0], c));
  int iter = 0;

  uint64_t m = p.n;
  const fe *a = w;
  if (open) goto opening;
  {
  // 2. evaluation point and its eq table.
  off = lay.rec(T_EVAL_POINT, logn, 16);
  RUN(PC_PROTOCOL, 1, k_point<<<B, 32, 0, s>>>(st, logn, tr, off, trs));
  // eq table E_0 of z_1..z_{logn-1} (the eq factor of variable 0 is kept apart)
  RUN(PC_BETA, 1, beta_launch(st->z + 1, logn - 1, p.vb[0], s, B, sts, p.bs_v));

  // 3. sumcheck of sum w(x) eq(z, x): w is folded each round, the eq vector
  //    is represented by the shrinking tables E_i (vb ping-pong) and the
  //    prefix product epre (k_sc_round_eq).
  uint64_t off_claim = lay.rec(T_CLAIM, 1, 16);
  int pp = 0, ep = 0;  // va ping-pong for w, vb ping-pong for E
  bool tail_done = false;
  uint64_t as = p.bs_w;  // per-proof stride of a (the witness, then va)
  for (int i = 0; i < logn; i++) {
    if (i >= 1 && m <= (uint64_t)kScTailMax) {
      // the remaining rounds and the final fold in one CTA
      const uint64_t op0 = lay.rec(T_SC_POLY, 3, 16);
      for (int r = i; r < logn; r++) {
        const uint64_t op = r == i ? op0 : lay.rec(T_SC_POLY, 3, 16);
        const uint64_t oc = lay.rec(T_SC_CHALLENGE, 1, 16);
        if (op != op0 + 80ull * (uint64_t)(r - i) || oc != op + 56) throw ArgError("prover: sumcheck record layout");
      }
      off = lay.rec(T_SC_FINAL, 2, 16);
      BStr tb;
      tb.s[0] = as;
      tb.s[1] = p.bs_v;
      tb.s[2] = trs;
      RUN(PC_SUMCHECK, 1,
          (k_sc_tail<<<B, kScTailThreads, sizeof(fe) * (kScTailMax + kScTailMax / 2), s>>>(st, a, p.vb[ep], (int)m, i,
                                                                                         logn, tr, op0, off, tb)));
      tail_done = true;
      break;
    }
    uint64_t off_poly = lay.rec(T_SC_POLY, 3, 16);
    uint64_t off_chal = lay.rec(T_SC_CHALLENGE, 1, 16);
    int blocks;
    // strides of (a, E, chal, a2, E2, partial)
    BStr es;
    es.s[0] = as;
    es.s[1] = p.bs_v;
    es.s[2] = sts;
    es.s[3] = p.bs_v;
    es.s[4] = p.bs_v;
    es.s[5] = p.bs_part;
    if (i == 0) {
      blocks = sc_blocks(m / 2);
      RUN(PC_SUMCHECK, 1,
          sc_eq_step_launch(a, p.vb[0], m, nullptr, nullptr, nullptr, true, p.partial, blocks, s, B, es));
    } else {
      blocks = sc_blocks(m / 4);
      fe *a2 = p.va[pp];
      RUN(PC_SUMCHECK, 1,
          sc_eq_step_launch(a, p.vb[ep], m, &st->chal[i - 1], a2, p.vb[ep ^ 1], true, p.partial, blocks, s, B, es));
      a = a2;
      as = p.bs_v;
      pp ^= 1;
      ep ^= 1;
      m /= 2;
    }
    RUN(PC_PROTOCOL, 1,
        k_sc_round_eq<<<B, 256, 0, s>>>(p.partial, blocks, st, i, tr, i == 0 ? (int64_t)off_claim : -1, off_poly,
                                        off_chal, p.bs_part, trs));
  }
  if (!tail_done) {
    fe *a2 = p.va[pp];
    BStr es;
    es.s[0] = as;
    es.s[1] = p.bs_v;
    es.s[2] = sts;
    es.s[3] = p.bs_v;
    es.s[4] = p.bs_v;
    es.s[5] = p.bs_part;
    RUN(PC_SUMCHECK, 1,
        sc_eq_step_launch(a, p.vb[ep], m, &st->chal[logn - 1], a2, nullptr, false, p.partial, 1, s, B, es));
    off = lay.rec(T_SC_FINAL, 2, 16);
    BStr fs;
    fs.s[0] = p.bs_v;
    fs.s[2] = trs;
    RUN(PC_PROTOCOL, 1, k_sc_final<<<B, 32, 0, s>>>(st, a2, nullptr, tr, off, fs));
    pp ^= 1;
  }
  }
opening:

  // 4. WHIR open of (v1[0], chal): b = precompute_beta(chal), arr = w.
  //    Three chains: folds and beta updates on s, commits on c, queries
  //    and the running claim K on q.  The folded polynomials are written
  //    once each (p.arr), so the commits read them while s moves on; a
  //    commit reuses a codeword/tree buffer only after the query that
  //    opened its previous content.
  // b = precompute_beta(chal) has tensor structure: for the first
  // iteration only the eq table E2 of chal[2..] is formed (a quarter of b)
  const bool eq_first = logn >= 4;
  RUN(PC_BETA, 1,
      eq_first ? beta_launch(st->chal + 2, logn - 2, p.beta, s, B, sts, p.bs_beta)
               : beta_launch(st->chal, logn, p.beta, s, B, sts, p.bs_beta));
  if (!dry) GBZ_CUDA(cudaStreamWaitEvent(s, p.ev_sched, 0));  // round challenges
  a = w;
  const fe *b = p.beta;
  uint64_t ast = p.bs_w, bst = p.bs_beta;  // per-proof strides of a and b
  m = p.n;
  uint64_t cur = (uint64_t)p.rate;
  fe *arr_next = p.arr;
  for (;;) {
    if (iter >= ProofPlan::kMaxIter) throw ArgError("prover: too many WHIR iterations");
    const int l = whir_query_count((int)cur);
    const uint64_t NL = 2 * cur * (m / 4);
    if (2 * NL != L) throw ArgError("prover: WHIR codeword lengths must halve");
    // both rounds in one pass over (a, b): their challenges were drawn up
    // front; arr_{t+1} goes to its own slot of p.arr, b to vb[(t + 1) mod 2]
    // (never the buffer it is read from)
    uint64_t op = lay.rec(T_WHIR_POLY, 3, 16), oc = lay.rec(T_WHIR_CHALLENGE, 1, 16);
    const uint64_t op1 = lay.rec(T_WHIR_POLY, 3, 16), oc1 = lay.rec(T_WHIR_CHALLENGE, 1, 16);
    fe *bd = p.vb[(iter + 1) & 1];
    const int blocks = sc_blocks(m / 4);
    if (iter == 0 && eq_first) {
      BStr fb;  // (a, E2, c, chal0, chal1, a4, b4, partial0, partial1)
      fb.s[0] = ast;
      fb.s[1] = bst;
      fb.s[2] = sts;
      fb.s[3] = sts;
      fb.s[4] = sts;
      fb.s[5] = p.bs_arr;
      fb.s[6] = p.bs_v;
      fb.s[7] = p.bs_part;
      fb.s[8] = p.bs_part;
      RUN(PC_SUMCHECK, 1,
          sc_fold2_eq_launch(a, b, m, st->chal, &st->wr[iter][0], &st->wr[iter][1], arr_next, bd, p.partial,
                             p.partial2, blocks, s, B, fb));
    } else {
      BStr fb;  // (a, b, chal0, chal1, a4, b4, partial0, partial1)
      fb.s[0] = ast;
      fb.s[1] = bst;
      fb.s[2] = sts;
      fb.s[3] = sts;
      fb.s[4] = p.bs_arr;
      fb.s[5] = p.bs_v;
      fb.s[6] = p.bs_part;
      fb.s[7] = p.bs_part;
      RUN(PC_SUMCHECK, 1,
          sc_fold2_launch(a, b, m, &st->wr[iter][0], &st->wr[iter][1], arr_next, bd, p.partial, p.partial2, blocks,
                          s, B, fb));
    }
    {
      // both round messages; the kernel also prepares this iteration's beta update
      UbPrep u{};
      if (!dry) {
        const NttTables &tnew = p.tables(ilog2(NL));
        u.l = l;
        u.lo = tnew.lo_fwd;
        u.hi = tnew.hi_fwd;
      }
      RUN(PC_PROTOCOL, 1,
          k_whir_rounds2_s<<<B, 256, 0, s>>>(p.partial, p.partial2, blocks, st, iter, tr, op, oc, op1, oc1, u,
                                             p.bs_part, trs));
    }
    a = arr_next;
    b = bd;
    ast = p.bs_arr;
    bst = p.bs_v;
    m /= 4;
    arr_next += m;
    if (!dry) GBZ_CUDA(cudaEventRecord(p.ev_fold[iter], s));
    // commit arr_{t+1} at rate 2*cur on c, once the query that opened the
    // buffer's previous codeword (iteration t-1) is done
    const int nci = cwi ^ 1;
    off = lay.rec(T_WHIR_ROOT, 1, 32);
    if (!dry) {
      GBZ_CUDA(cudaStreamWaitEvent(c, p.ev_fold[iter], 0));
      if (iter > 0) GBZ_CUDA(cudaStreamWaitEvent(c, p.ev_query[iter - 1], 0));
    }
    if (B > 1) {
      RUN_ON(c, PC_NTT, ntt_launch_count(ilog2(NL)),
             ntt_launch_rows(p.tables(ilog2(NL)), a, m, p.bs_arr / sizeof(fe), p.cw[nci], cw_s[nci] / sizeof(fe), B,
                             p.tmp, false, c));
    } else {
      RUN_ON(c, PC_NTT, ntt_launch_count(ilog2(NL)), ntt_launch(p.tables(ilog2(NL)), a, m, p.cw[nci], p.tmp, false, c));
    }
    off_root[iter + 1] = off;
    if (!dry) GBZ_CUDA(cudaEventRecord(p.ev_commit[iter + 1], c));
    // queries of iteration t on q: they open the codeword of commit t and
    // check K against this iteration's round messages
    const int depth = ilog2(L / 4);
    QueryArgs qa;
    qa.st = st;
    qa.cws = cw_s[cwi];
    qa.trs = trs;
    qa.cw = p.cw[cwi];
    qa.L = L;
    qa.NL = NL;
    qa.l = l;
    qa.tr = tr;
    qa.off_q = lay.rec(T_WHIR_QUERIES, l, 4);
    qa.off_rep = lay.rec(T_WHIR_REPLIES, l * kWhirK, 16);
    qa.off_ans = lay.rec(T_WHIR_ANSWERS, l, 16);
    qa.off_path = lay.rec(T_WHIR_PATHS, l * depth, 32);
    qa.off_comb = lay.rec(T_WHIR_COMBINE, l, 16);
    qa.off_K = lay.rec(T_WHIR_K, 1, 16);
    if (!dry) {
      const NttTables &told = p.tables(ilog2(L));
      qa.inv_lo = told.lo_inv;
      qa.inv_hi = told.hi_inv;
      qa.new_lo = nullptr;
      qa.new_hi = nullptr;
      const fe om_inv = finv(root_of_unity(ilog2(L)));
      qa.step0 = fpow(om_inv, L / kWhirK);
      qa.len_inv = finv(fe_make(kWhirK, 0));
      // the codeword it opens, and this iteration's round messages (for
      // iteration 0 also K = v1[0], set before on s)
      GBZ_CUDA(cudaStreamWaitEvent(q, p.ev_commit[iter], 0));
      GBZ_CUDA(cudaStreamWaitEvent(q, p.ev_fold[iter], 0));
    }
    RUN_ON(q, PC_MERKLE, 1, k_merkle_root_b<<<B, 32, 0, q>>>(qa.cw, qa.cws, depth, tr, trs, off_root[iter]));
    RUN_ON(q, PC_QUERY, 1, k_whir_query_s<<<B, kMaxQueries, 0, q>>>(qa, iter));
    {
      const uint64_t hashes = (uint64_t)l * depth;  // depth >= 2: every queried codeword has 16+ entries
      RUN_ON(q, PC_QUERY, 1,
             k_whir_paths_chain<<<dim3((unsigned)((hashes + 127) / 128), B), 128, 0, q>>>(
                 qa.cw, L / 4, l, tr, qa.off_q, qa.off_path, qa.cws, trs));
      if (!dry && hashes == 0) throw ArgError("prover: empty authentication paths");
    }
    if (!dry) GBZ_CUDA(cudaEventRecord(p.ev_query[iter], q));
    // update_betas on s: b[j] += sum_i c_i omega_NL^{q_i j} is the forward
    // transform of a vector with l nonzeros.  When l * |b| exceeds a few
    // transform lengths, the sparse transform is cheaper than the direct
    // sums.  The query exponents q_i * (whir_k NL / L) are even (NL = L / 2),
    // so omega_NL^{2 q_i j} = omega_{NL/2}^{q_i j}: the sparse transform runs
    // at half the codeword length on the unscaled positions.
    static_assert(kWhirK == 4, "update_betas: exponent scale 2 assumes folding by 4 with NL = L / 2");
    if (update_betas_by_transform(l, m, NL / 2)) {
      // one sparse transform per proof of a batch
      RUN(PC_UPDATE_BETAS, 2 * B, for (int pb = 0; pb < B; pb++) {
        ntt_sparse_accumulate(p.tables(ilog2(NL) - 1), st[pb].q, st[pb].comb, l,
                              reinterpret_cast<fe *>(reinterpret_cast<char *>(bd) + p.bs_v * pb), m,
                              reinterpret_cast<fe *>(reinterpret_cast<char *>(p.tmp2) + p.bs_tmp2 * pb), s, 1);
      });
    } else {
      RUN(PC_UPDATE_BETAS, 2, update_betas_launch(bd, m, st, l, p.ub_scratch, s, B, p.bs_v, p.bs_ub));
    }
    cwi = nci;
    L = NL;
    cur *= 2;
    iter++;
    if (m <= (uint64_t)kWhirK) break;
  }
  uint64_t off_poly = lay.rec(T_FINAL_POLY, (uint32_t)m, 16);
  uint64_t off_point = lay.rec(T_FINAL_POINT, ilog2(m), 16);
  uint64_t off_eval = lay.rec(T_FINAL_EVAL, 1, 16);
  {
    BStr fb;  // (arr, b, tr)
    fb.s[0] = ast;
    fb.s[1] = bst;
    fb.s[2] = trs;
    RUN(PC_PROTOCOL, 1, k_final_b<<<B, 32, 0, s>>>(st, a, b, (int)m, tr, off_poly, off_point, off_eval, fb));
  }
  // root of the last commitment (never opened) on the query stream
  if (!dry) GBZ_CUDA(cudaStreamWaitEvent(q, p.ev_commit[iter], 0));
  RUN_ON(q, PC_MERKLE, 1,
         k_merkle_root_b<<<B, 32, 0, q>>>(p.cw[cwi], cw_s[cwi], ilog2(L / 4), tr, trs, off_root[iter]));
  if (!dry) {  // join the commit and query chains
    GBZ_CUDA(cudaEventRecord(p.ev_root_tail, q));
    GBZ_CUDA(cudaStreamWaitEvent(s, p.ev_commit[iter], 0));
    GBZ_CUDA(cudaStreamWaitEvent(s, p.ev_root_tail, 0));
  }
#undef RUN
#undef RUN_ON
}

void Profiler::begin(int cat, cudaStream_t s) {
  auto &v = ev[cat];
  if (used[cat] == v.size()) {
    cudaEvent_t a, b;
    GBZ_CUDA(cudaEventCreate(&a));
    GBZ_CUDA(cudaEventCreate(&b));
    v.push_back({a, b});
  }
  GBZ_CUDA(cudaEventRecord(v[used[cat]].first, s));
  open_cat = cat;
}

void Profiler::end(cudaStream_t s) {
  auto &v = ev[open_cat];
  GBZ_CUDA(cudaEventRecord(v[used[open_cat]].second, s));
  used[open_cat]++;
  open_cat = -1;
}

void Profiler::read(double ms[PC_COUNT], int counts[PC_COUNT]) {
  for (int c = 0; c < PC_COUNT; c++) {
    double t = 0;
    for (size_t i = 0; i < used[c]; i++) {
      float x = 0;
      GBZ_CUDA(cudaEventSynchronize(ev[c][i].second));
      GBZ_CUDA(cudaEventElapsedTime(&x, ev[c][i].first, ev[c][i].second));
      t += x;
    }
    ms[c] = t;
    if (counts) counts[c] = (int)used[c];
  }
}

Profiler::~Profiler() {
  for (int c = 0; c < PC_COUNT; c++)
    for (auto &e : ev[c]) {
      cudaEventDestroy(e.first);
      cudaEventDestroy(e.second);
    }
}

namespace {
__global__ void k_set_seed(ProofState *st, uint32_t seed) {
  if (threadIdx.x == 0) st->seed_in = seed;
}
struct SeedChunk {
  uint32_t v[64];
};
__global__ void k_set_seeds(ProofState *st, SeedChunk c, int count) {
  if ((int)threadIdx.x < count) st[threadIdx.x].seed_in = c.v[threadIdx.x];
}
}  // namespace

void set_seed_launch(ProofPlan &p, uint32_t seed, cudaStream_t s) {
  k_set_seed<<<1, 32, 0, s>>>(p.st, seed);
  GBZ_CUDA(cudaGetLastError());
}

void set_seeds_launch(ProofPlan &p, const uint32_t *seeds, int count, cudaStream_t s) {
  for (int o = 0; o < count; o += 64) {
    SeedChunk c{};
    const int k = std::min(64, count - o);
    for (int i = 0; i < k; i++) c.v[i] = seeds[o + i];
    k_set_seeds<<<1, 64, 0, s>>>(p.st + o, c, k);
    GBZ_CUDA(cudaGetLastError());
  }
}

void launch_proof_graph(ProofPlan &p, const fe *w, uint32_t prng_seed, cudaStream_t s) {
  ProofGraph *g = nullptr;
  for (auto &e : p.graphs)
    if (e.w == w) g = &e;
  if (!g) {
    constexpr size_t kMaxGraphs = 4;
    if (p.graphs.size() >= kMaxGraphs) {  // drop the least recently used
      size_t lru = 0;
      for (size_t i = 1; i < p.graphs.size(); i++)
        if (p.graphs[i].last_use < p.graphs[lru].last_use) lru = i;
      GBZ_CUDA(cudaStreamSynchronize(s));
      cudaGraphExecDestroy(p.graphs[lru].exec);
      cudaGraphDestroy(p.graphs[lru].graph);
      p.graphs.erase(p.graphs.begin() + lru);
    }
    ProofGraph ng;
    ng.w = w;
    GBZ_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue_proof(p, w, prng_seed, s, false, false);
    } catch (...) {
      cudaGraph_t tmp = nullptr;
      cudaStreamEndCapture(s, &tmp);
      if (tmp) cudaGraphDestroy(tmp);
      throw;
    }
    GBZ_CUDA(cudaStreamEndCapture(s, &ng.graph));
    // the k_init node carries the seed
    size_t count = 0;
    GBZ_CUDA(cudaGraphGetNodes(ng.graph, nullptr, &count));
    std::vector<cudaGraphNode_t> nodes(count);
    GBZ_CUDA(cudaGraphGetNodes(ng.graph, nodes.data(), &count));
    for (auto nd : nodes) {
      cudaGraphNodeType ty;
      GBZ_CUDA(cudaGraphNodeGetType(nd, &ty));
      if (ty != cudaGraphNodeTypeKernel) continue;
      cudaKernelNodeParams kp{};
      GBZ_CUDA(cudaGraphKernelNodeGetParams(nd, &kp));
      if (kp.func == reinterpret_cast<void *>(k_init)) {
        ng.init_node = nd;
        ng.init_params = kp;
        break;
      }
    }
    if (!ng.init_node) {
      cudaGraphDestroy(ng.graph);
      throw ArgError("prover graph: initial node not found");
    }
    GBZ_CUDA(cudaGraphInstantiate(&ng.exec, ng.graph, 0));
    p.graphs.push_back(ng);
    g = &p.graphs.back();
  }
  g->last_use = ++p.graph_tick;
  ProofState *st = p.st;
  uint32_t seed_v = prng_seed;
  int flag = 0;
  void *args[3] = {&st, &seed_v, &flag};
  cudaKernelNodeParams kp = g->init_params;
  kp.kernelParams = args;
  kp.extra = nullptr;
  GBZ_CUDA(cudaGraphExecKernelNodeSetParams(g->exec, g->init_node, &kp));
  GBZ_CUDA(cudaGraphLaunch(g->exec, s));
}

uint64_t plan_bytes(int logn, int rate, int batch) {
  const uint64_t n = 1ull << logn, L = n * (uint64_t)rate;
  uint64_t b = sizeof(fe) * (n + L + L / 2 + L + L / 2 + 5 * (n / 2) + n);
  b += sizeof(fe) * (6 * (uint64_t)sc_blocks(n / 2) + kUpdateBetasScratch) + sizeof(ProofState);
  b *= (uint64_t)batch;
  b += 64ull << 20;  // transcripts, twiddle tables and allocation granularity (upper bound)
  b += (uint64_t)batch << 20;
  return b;
}

uint32_t plan_error_flags(ProofPlan &p, cudaStream_t s) {
  uint32_t e = 0;
  GBZ_CUDA(cudaMemcpyAsync(&e, &p.st->error, 4, cudaMemcpyDeviceToHost, s));
  GBZ_CUDA(cudaStreamSynchronize(s));
  return e;
}

}  // namespace gbz
