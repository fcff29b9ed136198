// The leader's side of PCS_open_new after the parties' rounds, on the device.
//
// In the reference the leader (rank 0) ends the collaborative opening alone:
// in every delegate check after the first it commits to the gathered
// segments with WHIR, draws extension queries and proves the folding and
// the extension of the segments (delegate_checks, coPCS.cpp:770-831); then
// it decodes and unpacks the parties' final data, checks the claim,
// aggregates the delegation claims and opens them with one WHIR opening,
// checks the final evaluation and delegates the evaluation of the betas
// (coPCS.cpp:1697-1753).  Every randomness of that tail comes from the
// leader's glibc generator (F::_random(), rand()), never from the
// Fiat-Shamir chain, and depends on the sizes alone; the tail therefore
// runs after the parties' rounds as one stream of launches that draws from
// one device-resident generator in the reference's order.
//
// The delegation sumchecks (quadruple_sumcheck, _cubic_sumcheck,
// _quadratic_sumcheck of delegate_protocol.cpp) run on the round-form
// kernels of gbz_rounds.cu with their challenges drawn ahead: each draws
// one F::_random() per coefficient and keeps the last (the rounds' own
// messages never enter the generator).  The WHIR opening is the batch
// opening's walk for one polynomial starting from the zero-leaf tree that
// aggregate_commitments installs.
#include <algorithm>
#include <cstring>
#include <map>

#include "gbz_batch_open.cuh"
#include "gbz_copcs.cuh"
#include "gbz_pcs_leader.cuh"
#include "gbz_rounds.cuh"
#include "gbz_whir_aggr.cuh"

namespace gbz {

namespace {

// Transcript tags of the tail (include/gbz.h).
enum : uint32_t {
  T_D_ROOT = 46, T_D_QUERIES = 47, T_D_POLYS = 48, T_D_FINAL = 49, T_D_CLAIM = 50, T_D_OPEN = 51,
  T_D_EXT_CLAIM = 52, T_L_UNPACKED = 53, T_L_WHIR_CLAIM = 54, T_L_RC = 55, T_L_BETA_Y = 56, T_L_EVALS = 57,
  T_L_LAG_EVALS = 69
};

constexpr int kT = 256;
constexpr int kMaxTailIter = 16;

unsigned nblk(uint64_t n, unsigned t = kT) { return (unsigned)std::max<uint64_t>(1, (n + t - 1) / t); }

__device__ __forceinline__ int ilog2_dev(uint64_t x) { return 63 - __clzll((long long)x); }

__device__ __forceinline__ fe get_fe(const uint8_t *tr, uint64_t off) {
  const uint32_t *p = reinterpret_cast<const uint32_t *>(tr + off);
  return fe_make((uint64_t)p[0] | ((uint64_t)p[1] << 32), (uint64_t)p[2] | ((uint64_t)p[3] << 32));
}

__device__ __forceinline__ fe pow_tab(const fe *lo, const fe *hi, uint64_t e) {
  return fmul(lo[e & 4095u], hi[e >> 12]);
}

// Sum of one value per thread over a block of kT threads; valid in thread 0.
__device__ fe block_sum_fe(fe v) {
  __shared__ fe red[kT];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = kT / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] = fadd(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  const fe r = red[0];
  __syncthreads();
  return r;
}

// ---- the generator ---------------------------------------------------------
// The tail's draws in the reference's order, one thread: F::_random()
// (fieldElement.cpp:119-125) into the arena, rand() % mod (coPCS.cpp:789,
// Whir.cpp:574-576) into the transcript, the state the WHIR opening starts
// from into st->prng, the calls the opening makes itself skipped (their
// end state into after_walk), and the final state.
__global__ void k_draw_script(glibc_prng g0, const DrawOp *ops, int nops, fe *arena, uint8_t *tr, ProofState *st,
                              glibc_prng *after_walk, glibc_prng *final_state) {
  __shared__ glibc_prng g;  // dynamically indexed table: work on a shared copy
  if (threadIdx.x) return;
  g = g0;
  for (int k = 0; k < nops; k++) {
    const DrawOp o = ops[k];
    if (o.kind == DRAW_FIELDS) {
      for (int i = 0; i < o.count; i++) arena[o.off + i] = prng_field(g);
    } else if (o.kind == DRAW_INTS) {
      uint32_t *q = reinterpret_cast<uint32_t *>(tr + o.off);
      for (int i = 0; i < o.count; i++) q[i] = (uint32_t)(prng_next(g) % (int32_t)o.mod);
    } else if (o.kind == DRAW_STATE) {
      st->prng = g;
    } else {
      for (int i = 0; i < o.count; i++) (void)prng_next(g);
      *after_walk = g;
    }
  }
  *final_state = g;
}

// The WHIR opening drew as many values as the script skipped for it.
__global__ void k_prng_check(const ProofState *st, const glibc_prng *expect, uint32_t *flags) {
  if (threadIdx.x) return;
  bool same = st->prng.f == expect->f && st->prng.r == expect->r;
  for (int i = 0; i < 31; i++) same = same && st->prng.tbl[i] == expect->tbl[i];
  if (!same) atomicOr(flags, LF_WHIR);
}

__global__ void k_tail_init(ProofState *st, glibc_prng g, uint32_t *flags) {
  if (threadIdx.x) return;
  st->prng = g;
  st->K = fe_zero();
  st->fs = fe_zero();
  st->y = fe_zero();
  st->error = 0;
  *flags = 0;
}

// ---- the delegation sumchecks ------------------------------------------------
// Round message H of the partials, the check H(0) + H(1) = y (flag `bit`),
// the challenge drawn ahead, y = H(challenge).
__global__ void k_sc_finish(const fe *partial, int blocks, int nc, fe *y, const fe *draw, fe *ch, int round,
                            uint32_t *flags, uint32_t bit, uint8_t *tr, uint64_t off_polys) {
  __shared__ fe red[kMaxFormCoeffs][kT];
  fe acc[kMaxFormCoeffs];
  for (int k = 0; k < kMaxFormCoeffs; k++) acc[k] = fe_zero();
  for (int i = threadIdx.x; i < blocks; i += kT)
    for (int k = 0; k < nc; k++) acc[k] = fadd(acc[k], partial[(uint64_t)i * nc + k]);
  for (int k = 0; k < kMaxFormCoeffs; k++) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int w = kT / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < kMaxFormCoeffs; k++) red[k][threadIdx.x] = fadd(red[k][threadIdx.x], red[k][threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x) return;
  // coefficients highest degree first: H(0) + H(1) = 2 c_last + the others
  fe s = red[nc - 1][0];
  for (int k = 0; k < nc; k++) s = fadd(s, red[k][0]);
  if (bit && !fe_eq(s, *y)) atomicOr(flags, bit);
  for (int k = 0; k < nc; k++) put_fe(tr, off_polys + 16ull * ((uint64_t)round * nc + k), red[k][0]);
  const fe c = *draw;
  ch[round] = c;
  fe v = red[0][0];
  for (int k = 1; k < nc; k++) v = fadd(fmul(v, c), red[k][0]);
  *y = v;
}

__global__ void k_set(fe *dst, const fe *src) {
  if (threadIdx.x == 0) *dst = *src;
}

// ---- prove_multi_folding (delegate_protocol.cpp:147-250) ---------------------
// One CTA per segment t < S: get_RS_multifold_segment (coPCS_utils.cpp:268-331)
// of segment t (it does not depend on the query position: its twiddles
// start at 1), the powers (omega_n^-1)^(q_t j), and the other two vectors of
// the quadruple sumcheck: V3 = L in every block, V4 = b1[t].  Rows t >= l
// (pad_vector) are zero in V1 and V2.  twd[k] = omega_d^-k.
__global__ void k_pmf_vectors(const fe *seg, const int32_t *qpos, int l, int d, int logd, const fe *twd, fe wn_inv,
                              const fe *L, const fe *b1, fe *V1, fe *V2, fe *V3, fe *V4) {
  extern __shared__ fe sh[];
  fe *X = sh, *Y = sh + d;
  __shared__ fe wt;
  const int t = blockIdx.x;
  const uint64_t base = (uint64_t)t * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    V3[base + j] = L[j];
    V4[base + j] = b1[t];
  }
  if (t >= l) {
    for (int j = threadIdx.x; j < d; j += blockDim.x) V1[base + j] = V2[base + j] = fe_zero();
    return;
  }
  if (threadIdx.x == 0) wt = fpow(wn_inv, (uint64_t)(uint32_t)qpos[t]);
  // level 0: group j < d/2 holds (s_j + s_{j+d/2}, omega_d^-j (s_j - s_{j+d/2}))
  for (int j = threadIdx.x; j < d / 2; j += blockDim.x) {
    const fe a = seg[base + j], b = seg[base + j + d / 2];
    X[2 * j] = fadd(a, b);
    X[2 * j + 1] = fmul(twd[j], fsub(a, b));
  }
  __syncthreads();
  // level i: group j of width 2w joins old groups j and j + J, twiddle omega_d^-(w j)
  for (int i = 1; i < logd; i++) {
    const int w = 1 << i, J = d >> (i + 1);
    for (int e = threadIdx.x; e < d / 2; e += blockDim.x) {
      const int j = e / w, k = e % w;
      const fe p = X[j * w + k], q = X[(j + J) * w + k];
      Y[j * 2 * w + k] = fadd(p, q);
      Y[j * 2 * w + k + w] = fmul(twd[((uint64_t)w * j) & (uint64_t)(d - 1)], fsub(p, q));
    }
    __syncthreads();
    fe *tt = X;
    X = Y;
    Y = tt;
  }
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    V1[base + j] = X[j];
    V2[base + j] = fpow(wt, (uint64_t)j);
  }
}

// out = scale * sum_{t < n} a[t] b[t] (one CTA), also into *y2 when given.
__global__ void k_dot(const fe *a, const fe *b, uint64_t n, fe scale, fe *out) {
  fe acc = fe_zero();
  for (uint64_t t = threadIdx.x; t < n; t += kT) acc = fadd(acc, fmul(a[t], b[t]));
  acc = block_sum_fe(acc);
  if (threadIdx.x == 0) *out = fmul(scale, acc);
}

// The verifier's checks after the quadruple sumcheck (delegate_protocol.cpp:197-229):
// fin[1] = sum_t b12[t] prod_j (1 - r11_j + r11_j w_t^(2^j)), fin[2] = <b11, L>,
// fin[3] = prod_i eq(r12_i, r1_i).  ch = r11 (logd) then r12 (logS).
__global__ void k_pmf_checks(const fe *fin, const fe *ch, int logd, int logS, const fe *r1, const fe *b12,
                             const fe *b11, const fe *L, const int32_t *qpos, int l, int d, fe wn_inv,
                             uint32_t *flags) {
  fe acc = fe_zero();
  for (int t = threadIdx.x; t < l; t += kT) {
    fe w = fpow(wn_inv, (uint64_t)(uint32_t)qpos[t]), c = fe_one();
    for (int j = 0; j < logd; j++) {
      c = fmul(c, fadd(fsub(fe_one(), ch[j]), fmul(ch[j], w)));
      w = fmul(w, w);
    }
    acc = fadd(acc, fmul(b12[t], c));
  }
  acc = block_sum_fe(acc);
  fe acc2 = fe_zero();
  for (int i = threadIdx.x; i < d; i += kT) acc2 = fadd(acc2, fmul(b11[i], L[i]));
  acc2 = block_sum_fe(acc2);
  if (threadIdx.x) return;
  uint32_t bad = 0;
  if (!fe_eq(acc, fin[1])) bad = 1;
  if (!fe_eq(acc2, fin[2])) bad = 1;
  fe p = fe_one();
  for (int i = 0; i < logS; i++) {
    const fe a = ch[logd + i], b = r1[i];
    p = fmul(p, fadd(fmul(fsub(fe_one(), a), fsub(fe_one(), b)), fmul(a, b)));
  }
  if (!fe_eq(p, fin[3])) bad = 1;
  if (bad) atomicOr(flags, LF_DELEGATION);
}

// out[j] = sum_{t < l} w[t] seg[t d + j] for j < d (one CTA per j).
__global__ void k_seg_comb(const fe *seg, const fe *w, int l, int d, fe *out) {
  const int j = blockIdx.x;
  fe acc = fe_zero();
  for (int t = threadIdx.x; t < l; t += kT) acc = fadd(acc, fmul(w[t], seg[(uint64_t)t * d + j]));
  acc = block_sum_fe(acc);
  if (threadIdx.x == 0) out[j] = acc;
}

// get_RS_multifold_reduced_matrix (coPCS_utils.cpp:235-266) over d entries:
// rm[j] = (1 - r_0 +- omega_d^-j' r_0) prod_{i >= 1} (1 - r_i + omega_d^-(2^i j') r_i), j' = j mod d/2,
// the sign negative in the upper half.
__global__ void k_reduced_matrix(const fe *r, int logd, int d, const fe *twd, fe *out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d) return;
  const int h = j & (d / 2 - 1);
  const fe w0 = fmul(twd[h], r[0]);
  fe v = fsub(fe_one(), r[0]);
  v = j < d / 2 ? fadd(v, w0) : fsub(v, w0);
  for (int i = 1; i < logd; i++)
    v = fmul(v, fadd(fsub(fe_one(), r[i]), fmul(twd[((uint64_t)h << i) & (uint64_t)(d - 1)], r[i])));
  out[j] = v;
}

// evaluate_vector (utils.cpp:1201-1214) of n <= 2^13 entries in one CTA:
// folds by r[0], r[1], ... through two scratch halves.
__global__ void k_eval(const fe *v, int logn, const fe *r, fe *s0, fe *s1, fe *out) {
  const int n = 1 << logn;
  const fe *src = v;
  fe *dst = s0;
  for (int i = 0; i < logn; i++) {
    const int half = n >> (i + 1);
    const fe ri = r[i], om = fsub(fe_one(), ri);
    for (int j = threadIdx.x; j < half; j += blockDim.x) dst[j] = fadd(fmul(om, src[2 * j]), fmul(ri, src[2 * j + 1]));
    __syncthreads();
    src = dst;
    dst = dst == s0 ? s1 : s0;
  }
  if (threadIdx.x == 0) *out = src[0];
}

__global__ void k_check_eq(const fe *a, const fe *b, uint32_t *flags, uint32_t bit) {
  if (threadIdx.x == 0 && !fe_eq(*a, *b)) atomicOr(flags, bit);
}

// The claim kept for the WHIR aggregation: (value, r_sum ++ r12, zeros up to
// pad) (delegate_protocol.cpp:246-249, coPCS.cpp:843-853).
__global__ void k_claim(const fe *value, const fe *ra, int na, const fe *rb, int nb, int pad, fe *claim, uint8_t *tr,
                        uint64_t off) {
  const int k = threadIdx.x;
  if (k > pad) return;
  fe v;
  if (k == 0) v = *value;
  else if (k - 1 < na) v = ra[k - 1];
  else if (k - 1 - na < nb) v = rb[k - 1 - na];
  else v = fe_zero();
  claim[k] = v;
  put_fe(tr, off + 16ull * k, v);
}

// ---- prove_extension (delegate_protocol.cpp:369-429) ---------------------------
// o_t = E[t][q_t], the one-hot rows V2 and the weights V3[t][j] = b[t].
__global__ void k_pe_vectors(const fe *E, const int32_t *q2, int l, uint64_t C0, const fe *b, fe *o, fe *V2, fe *V3,
                             uint64_t total, uint8_t *tr, uint64_t off_o) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const uint64_t t = g / C0, j = g % C0;
  V3[g] = b[t];
  const bool hit = t < (uint64_t)l && j == (uint64_t)(uint32_t)q2[t];
  V2[g] = hit ? fe_one() : fe_zero();
  if (hit) {
    const fe v = E[g];
    o[t] = v;
    put_fe(tr, off_o + 16 * t, v);
  }
}

// Checks 5 and 6 (delegate_protocol.cpp:397-410): fin[1] = sum_t b1[q_t] b2[t],
// fin[2] = prod_i eq(r2_i, r_i).
__global__ void k_pe_checks(const fe *fin, const fe *b1e, const fe *b2e, const int32_t *q2, int l, const fe *r2e,
                            const fe *r, int logS, uint32_t *flags) {
  fe acc = fe_zero();
  for (int t = threadIdx.x; t < l; t += kT) acc = fadd(acc, fmul(b1e[(uint32_t)q2[t]], b2e[t]));
  acc = block_sum_fe(acc);
  if (threadIdx.x) return;
  uint32_t bad = !fe_eq(acc, fin[1]);
  fe p = fe_one();
  for (int i = 0; i < logS; i++)
    p = fmul(p, fadd(fmul(fsub(fe_one(), r2e[i]), fsub(fe_one(), r[i])), fmul(r2e[i], r[i])));
  if (!fe_eq(p, fin[2])) bad = 1;
  if (bad) atomicOr(flags, LF_DELEGATION);
}

// phiGInit(phi, r, scale, n, false) (utils.cpp:1131-1165) over 2^n
// entries: phi[b] = scale prod_{m < n} (1 - r_m + r_m omega^(b 2^m)) for
// b < 2^(n-1), zero above; omega = omega_{2^n} from the tables (lo, hi).
// With nr < n the missing r_m are zero (their factor is 1).
__global__ void k_phi(const fe *r, int nr, int n, const fe *lo, const fe *hi, fe scale, fe *out) {
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, N = 1ull << n;
  if (b >= N) return;
  if (b >= N / 2) {
    out[b] = fe_zero();
    return;
  }
  fe v = scale;
  for (int m = 0; m < nr; m++) v = fmul(v, fadd(fsub(fe_one(), r[m]), fmul(r[m], pow_tab(lo, hi, (b << m) & (N - 1)))));
  out[b] = v;
}

// prove_fft's claim (delegate_protocol.cpp:131-143) extended by r2
// (:419-422): c = fin[1]; log2(rate) times c = c (1 - r_last)^-1 c, then the
// point without its last log2(rate) entries.
__global__ void k_ext_claim(const fe *fin, const fe *rpf, int npf, int lograte, const fe *r2e, int logS, uint8_t *tr,
                            uint64_t off) {
  if (threadIdx.x) return;
  fe c = fin[1];
  const fe inv = finv(fsub(fe_one(), rpf[npf - 1]));
  for (int i = 0; i < lograte; i++) c = fmul(c, fmul(inv, c));
  put_fe(tr, off, c);
  int k = 1;
  for (int i = 0; i < npf - lograte; i++) put_fe(tr, off + 16ull * k++, rpf[i]);
  for (int i = 0; i < logS; i++) put_fe(tr, off + 16ull * k++, r2e[i]);
}

// ---- the final steps (coPCS.cpp:1697-1752) ---------------------------------------
// Decoding: the first n entries of every party's inverse-transformed C' are its data.
__global__ void k_decode_check(const fe *dec, uint64_t cpl, const fe *data, uint64_t n, int N, uint32_t *flags) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (uint64_t)N * n) return;
  const uint64_t p = g / n, j = g % n;
  if (!fe_eq(dec[p * cpl + j], data[g])) atomicOr(flags, LF_DECODING);
}

// unpack_secret_share(., N/2, N) of the data and of B (one value per party),
// then K - sum final_poly final_B = 0 (final verification step 1).
__global__ void k_unpack_final(const fe *U, const fe *bcd, const fe *B, int N, const fe *K, fe *fp, fe *fB,
                               uint32_t *flags, uint8_t *tr, uint64_t off) {
  const int j = threadIdx.x;
  __shared__ fe prod[32];
  if (j < N / 2) {
    fe a = fe_zero(), b = fe_zero();
    for (int p = 0; p < N; p++) {
      a = fadd(a, fmul(U[j * N + p], bcd[p]));
      b = fadd(b, fmul(U[j * N + p], B[p]));
    }
    fp[j] = a;
    fB[j] = b;
    put_fe(tr, off + 16ull * j, a);
    put_fe(tr, off + 16ull * (N / 2 + j), b);
    prod[j] = fmul(a, b);
  }
  __syncthreads();
  if (j) return;
  fe k = *K;
  for (int i = 0; i < N / 2; i++) k = fsub(k, prod[i]);
  if (!fe_eq(k, fe_zero())) atomicOr(flags, LF_FINAL1);
}

// aggregate_claims' K (Whir.cpp:651-656) = sum_{a, c} bac[c] aac[a] Sums[a][c]
// (Sums row-major, R x R), into the opening's running claim.
__global__ void k_aggr_K(const fe *sums, const fe *ch, int R, ProofState *st, uint8_t *tr, uint64_t off_ch,
                         uint64_t off_K) {
  if (threadIdx.x) return;
  fe K = fe_zero();
  for (int a = 0; a < R; a++)
    for (int c = 0; c < R; c++) K = fadd(K, fmul(fmul(ch[c], ch[R + a]), sums[a * R + c]));
  st->K = K;
  put_fe(tr, off_K, K);
  for (int i = 0; i < 2 * R; i++) put_fe(tr, off_ch + 16ull * i, ch[i]);
}

struct ChalOffs {
  int n;
  uint64_t off[64];
};

// total_r of _Whir_Open (Whir.cpp:506-509): every round challenge, then the
// final point.
__global__ void k_gather_r(const uint8_t *tr, ChalOffs c, uint64_t off_point, int npoint, fe *out) {
  const int k = threadIdx.x;
  if (k < c.n) out[k] = get_fe(tr, c.off[k]);
  else if (k < c.n + npoint) out[k] = get_fe(tr, off_point + 16ull * (k - c.n));
}

// Verification step 1 of _Whir_Open (Whir.cpp:494-501): the final polynomial
// re-encoded at the final rate equals the last codeword.
__global__ void k_reencode_check(const fe *arr, int m, const fe *cw, uint64_t L, const fe *lo, const fe *hi,
                                 ProofState *st) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= L) return;
  fe v = fe_zero();
  for (int i = 0; i < m; i++) v = fadd(v, fmul(arr[i], pow_tab(lo, hi, ((uint64_t)i * j) & (L - 1))));
  if (!fe_eq(v, cw[j])) atomicOr(&st->error, 32u);
}

struct Step3Args {
  int iters, nr;                       // iterations; entries of total_r
  uint64_t off_q[kMaxTailIter], off_c[kMaxTailIter], NL[kMaxTailIter];
  int l[kMaxTailIter], skip[kMaxTailIter];  // queries; total_r entries erased before iteration i's identities
  int R, npt;                          // claims and their point length
  uint64_t off_eval, off_claim;
};

// Verification step 3 of _Whir_Open (Whir.cpp:511-539), printed by the
// reference when it fails: y = evaluate_vector(b, r_final) against the final
// claim plus the beta identities of the claims (weights bac) plus the
// omega identities of every iteration's scaled queries (weights c_i).
__global__ void k_whir_step3(const uint8_t *tr, Step3Args a, const fe *claims, const fe *bac, const fe *total_r,
                             uint32_t *flags) {
  fe acc = fe_zero();
  for (int it = 0; it < a.iters; it++) {
    const fe om = root_of_unity(ilog2_dev(a.NL[it]));
    for (int j = threadIdx.x; j < a.l[it]; j += kT) {
      const uint32_t q = reinterpret_cast<const uint32_t *>(tr + a.off_q[it])[j];
      fe w = fpow(om, 2ull * q), e = fe_one();
      for (int k = a.skip[it]; k < a.nr; k++) {
        e = fmul(e, fadd(fsub(fe_one(), total_r[k]), fmul(total_r[k], w)));
        w = fmul(w, w);
      }
      acc = fadd(acc, fmul(get_fe(tr, a.off_c[it] + 16ull * j), e));
    }
  }
  acc = block_sum_fe(acc);
  if (threadIdx.x) return;
  fe y_ = fadd(get_fe(tr, a.off_claim), acc);
  for (int c = 0; c < a.R; c++) {
    const fe *pt = claims + (uint64_t)c * (1 + a.npt) + 1;
    fe e = fe_one();
    for (int k = 0; k < a.npt; k++)
      e = fmul(e, fadd(fmul(fsub(fe_one(), pt[k]), fsub(fe_one(), total_r[k])), fmul(pt[k], total_r[k])));
    y_ = fadd(y_, fmul(bac[c], e));
  }
  if (!fe_eq(y_, get_fe(tr, a.off_eval))) atomicOr(flags, LF_WHIR_STEP3);
}

__global__ void k_put_claim_value(const fe *v, const fe *r, int nr, uint8_t *tr, uint64_t off) {
  const int k = threadIdx.x;
  if (k == 0) put_fe(tr, off, *v);
  else if (k <= nr) put_fe(tr, off + 16ull * k, r[k - 1]);
}

struct FinalRound {
  const fe *s;                  // the round's phase-3 challenge
  const int32_t *qp, *qpos;     // its queries
  int l, mul, div;              // positions rescaled by mul / div
  int nL;                       // Lagrange vectors of the later rounds
  const fe *L[8];
  int d[8];
  uint64_t rows;                // instance_size[i]
  int rate;                     // _rates[i][0]
};
struct FinalArgs {
  int nq, N;
  FinalRound q[8];
  const fe *fB, *b3, *r_first, *b2f, *rc;
  uint64_t off_rc;
};

// fast_eval_powers_y (New_PCS.cpp:582-605) per party p < N, at r_c: the
// inverse transform of length N/2 of the powers of omega_{2N}^(2p+1),
// evaluated as a polynomial in r_c.
__global__ void k_powers_y(int N, const fe *rcp, fe *py) {
  const int p = threadIdx.x;
  if (p >= N) return;
  const fe rc = *rcp;
  const int h = N / 2, lh = ilog2_dev((uint64_t)h);
  const fe w1 = fpow(root_of_unity(1 + ilog2_dev((uint64_t)N)), 2ull * p + 1);
  const fe winv = finv(root_of_unity(lh)), hinv = finv(fe_make((uint64_t)h, 0));
  fe acc = fe_zero(), rk = fe_one();
  for (int k = 0; k < h; k++) {
    fe c = fe_zero();
    const fe wk = fpow(winv, (uint64_t)k);
    fe x = fe_one(), wi = fe_one();
    for (int i = 0; i < h; i++) {
      c = fadd(c, fmul(x, wi));
      x = fmul(x, w1);
      wi = fmul(wi, wk);
    }
    acc = fadd(acc, fmul(rk, fmul(c, hinv)));
    rk = fmul(rk, rc);
  }
  py[p] = acc;
}

// The partial evaluations of the queries of the rounds before the last
// (coPCS.cpp:1733-1746): for query t of round r, s^(t+1)
// fast_eval_powers_x(L_{r+1..}, position, rows, rate) (New_PCS.cpp:610-634)
// times fast_eval_powers_y of its party.  One warp per query, its lanes over
// the Lagrange weights; terms[g] for the g-th query over all rounds.
__global__ void k_final_terms(FinalArgs a, const fe *py, fe *terms) {
  const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  int r = 0, t = g;
  while (r < a.nq && t >= a.q[r].l) t -= a.q[r++].l;
  if (r >= a.nq) return;
  const FinalRound &q = a.q[r];
  const uint64_t pos = (uint64_t)(uint32_t)q.qpos[t] * (uint64_t)q.mul / (uint64_t)q.div;
  fe om = fpow(root_of_unity(ilog2_dev((uint64_t)q.rate * q.rows)), pos), fx = fe_one();
  for (int k = 0; k < q.nL; k++) {
    if (k) om = fpow(om, (uint64_t)q.d[k - 1]);
    fe sum = fe_zero(), x = fpow(om, (uint64_t)lane);
    const fe step = fpow(om, 32);
    for (int j = lane; j < q.d[k]; j += 32) {
      sum = fadd(sum, fmul(q.L[k][j], x));
      x = fmul(x, step);
    }
    for (int d = 16; d > 0; d >>= 1) {
      fe u;
      u.re = __shfl_xor_sync(0xffffffffu, sum.re, d);
      u.im = __shfl_xor_sync(0xffffffffu, sum.im, d);
      sum = fadd(sum, u);
    }
    fx = fmul(fx, sum);
  }
  if (lane == 0) terms[g] = fmul(fmul(fpow(*q.s, (uint64_t)t + 1), fx), py[(uint32_t)q.qp[t]]);
}

// B_eval_claim = sum_i r_c^i final_B[i], b3(r_c), and the check
// r_first b2[0] b3(r_c) + sum of the terms = B_eval_claim ("final
// verification step", coPCS.cpp:1711-1752).
__global__ void k_final_eval(FinalArgs a, const fe *terms, int nterms, uint32_t *flags, uint8_t *tr) {
  fe acc = fe_zero();
  for (int g = threadIdx.x; g < nterms; g += kT) acc = fadd(acc, terms[g]);
  acc = block_sum_fe(acc);
  if (threadIdx.x) return;
  const fe rc = *a.rc;
  const int h = a.N / 2;
  fe be = fe_zero(), rk = fe_one();
  for (int i = 0; i < h; i++) {
    be = fadd(be, fmul(rk, a.fB[i]));
    rk = fmul(rk, rc);
  }
  fe b3c = fe_zero();
  rk = fe_one();
  for (int i = 0; i < a.N / 4; i++) {
    b3c = fadd(b3c, fmul(rk, a.b3[i]));
    rk = fmul(rk, rc);
  }
  const fe fin = fadd(fmul(fmul(*a.r_first, *a.b2f), b3c), acc);
  if (!fe_eq(fin, be)) atomicOr(flags, LF_FINAL);
  put_fe(tr, a.off_rc, rc);
  put_fe(tr, a.off_rc + 16, be);
}

// ---- delegate_beta_eval (delegate_protocol.cpp:431-504) ----------------------------
// L_vector: the tensor product of the rounds' Lagrange vectors, round 0 on
// the lowest index digits.
struct TensorArgs {
  int n;
  const fe *L[8];
  int logd[8];
};
__global__ void k_tensor(TensorArgs a, uint64_t total, fe *out) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  uint64_t x = g;
  fe v = fe_one();
  for (int k = 0; k < a.n; k++) {
    v = fmul(v, a.L[k][x & ((1ull << a.logd[k]) - 1)]);
    x >>= a.logd[k];
  }
  out[g] = v;
}

__global__ void k_mul(const fe *a, const fe *b, uint64_t n, fe *out) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n) out[g] = fmul(a[g], b[g]);
}

// The check "Error in delegating betas 1" (and delegate_lagrange_eval's
// second "Error in delegating betas 2"): prod_k evaluate_vector(L_k, r_k)
// against the sumcheck's value *fin for that tensor (bit: the flag); the
// evaluations go to the transcript.  scratch: 3/4 of the longest factor.
__global__ void k_beta_evals(TensorArgs a, const fe *r, const fe *fin, uint32_t bit, fe *scratch, uint32_t *flags,
                             uint8_t *tr, uint64_t off) {
  __shared__ fe ev[8];
  int base = 0;
  for (int k = 0; k < a.n; k++) {
    const int n = 1 << a.logd[k];
    fe *s0 = scratch, *s1 = scratch + n / 2;
    const fe *src = a.L[k];
    fe *dst = s0;
    for (int i = 0; i < a.logd[k]; i++) {
      const int half = n >> (i + 1);
      const fe ri = r[base + i], om = fsub(fe_one(), ri);
      for (int j = threadIdx.x; j < half; j += blockDim.x) dst[j] = fadd(fmul(om, src[2 * j]), fmul(ri, src[2 * j + 1]));
      __syncthreads();
      src = dst;
      dst = dst == s0 ? s1 : s0;
    }
    if (threadIdx.x == 0) ev[k] = src[0];
    __syncthreads();
    base += a.logd[k];
  }
  if (threadIdx.x) return;
  fe p = fe_one();
  for (int k = 0; k < a.n; k++) {
    put_fe(tr, off + 16ull * k, ev[k]);
    p = fmul(p, ev[k]);
  }
  if (!fe_eq(p, fin[0])) atomicOr(flags, bit);
}

// delegate_lagrange_eval's first "Error in delegating betas 2"
// (delegate_protocol.cpp:668-675): the multilinear extension of omega^j at
// the point, prod_i (1 - r_i + r_i omega^(2^i)), against the sumcheck's
// value of the omega vector.
__global__ void k_lag_omega(const fe *r, int n, fe omega, const fe *fin, uint32_t *flags) {
  if (threadIdx.x) return;
  fe p = fe_one();
  for (int i = 0; i < n; i++) {
    p = fmul(p, fadd(fsub(fe_one(), r[i]), fmul(r[i], omega)));
    omega = fmul(omega, omega);
  }
  if (!fe_eq(p, fin[2])) atomicOr(flags, LF_LAG2);
}

// "Error in delegating betas 3" (delegate_protocol.cpp:696-707): the ones
// vector's value plus the equality weights of its q zeroed entries
// Bs - q .. Bs - 1 at the point is one.
__global__ void k_lag_ones(const fe *fin, const fe *r, int n, uint64_t Bs, uint64_t q, uint32_t *flags) {
  __shared__ fe part[kT];
  fe acc = fe_zero();
  for (uint64_t i = Bs - q + threadIdx.x; i < Bs; i += blockDim.x) {
    fe b = fe_one();
    for (int j = 0; j < n; j++) b = fmul(b, (i >> j) & 1 ? r[j] : fsub(fe_one(), r[j]));
    acc = fadd(acc, b);
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x) return;
  fe sum = fin[2];
  for (int t = 0; t < (int)blockDim.x; t++) sum = fadd(sum, part[t]);
  if (!fe_eq(sum, fe_one())) atomicOr(flags, LF_LAG3);
}

// v[i] = 1 for i < m, 0 for m <= i < n.
__global__ void k_fill_prefix(fe *v, uint64_t n, uint64_t m) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n) v[g] = g < m ? fe_one() : fe_zero();
}

__global__ void k_put1(const fe *v, uint8_t *tr, uint64_t off) {
  if (threadIdx.x == 0) put_fe(tr, off, *v);
}

__global__ void k_whir_flags(const ProofState *st, uint32_t *flags) {
  if (threadIdx.x == 0 && st->error) atomicOr(flags, LF_WHIR);
}

// ---- host side ------------------------------------------------------------------------

// One walk over the tail: with tr == nullptr only the records are laid out.
struct Tail {
  LeaderResources &R;
  const LeaderInputs &in;
  ProofState *st;
  uint32_t *flags;
  uint8_t *tr;
  Layout &lay;
  bool dry;
  cudaStream_t s;
  std::vector<DrawOp> *script;  // the dry pass records the draws here
  const glibc_prng *after_walk; // the script's state after the WHIR opening's calls
  fe *arena;                    // the run reads them from here
  uint64_t arena_used;
  std::map<int, void *> slots;

  template <typename T>
  T *alloc(uint64_t n) {
    return dry ? nullptr : (T *)R.alloc(std::max<uint64_t>(n * sizeof(T), 16));
  }
  fe *zeros(uint64_t n) {
    fe *p = alloc<fe>(n);
    if (!dry) GBZ_CUDA(cudaMemsetAsync(p, 0, 16 * n, s));
    return p;
  }
  void check() {
    if (!dry) GBZ_CUDA(cudaGetLastError());
  }

  // A sumcheck of `form` over the vectors v (n entries each, read only)
  // from the claim *y: round i's challenge is draw[first + stride i]; ch
  // receives the challenges, fin the vectors' final values.
  void sumcheck(int form, const fe *const *v, uint64_t n, fe *y, const fe *draw, int first, int stride, fe *ch,
                fe *fin, uint32_t bit) {
    const int nv = form_vectors(form), nc = form_coeffs(form), rounds = ilog2(n);
    if (n < 2 || !is_pow2(n)) throw ArgError("pcs leader: sumcheck length must be a power of two >= 2");
    const uint64_t op = lay.rec(T_D_POLYS, (uint32_t)(rounds * nc), 16), of = lay.rec(T_D_FINAL, (uint32_t)nv, 16);
    if (dry) return;
    const int pb = round_blocks(n / 2);
    fe *partial = alloc<fe>((uint64_t)pb * nc);
    fe *buf[2][6] = {};
    for (int b = 0; b < 2; b++)
      for (int k = 0; k < nv; k++) buf[b][k] = alloc<fe>(std::max<uint64_t>(n / 2, 1));
    RoundArgs a{};
    for (int k = 0; k < nv; k++) a.in[k] = v[k];
    a.pairs = n / 2;
    a.partial = partial;
    form_step_launch(form, a, 0, round_blocks(a.pairs), s);
    k_sc_finish<<<1, kT, 0, s>>>(partial, round_blocks(a.pairs), nc, y, draw + first, ch, 0, flags, bit, tr, op);
    check();
    // rounds with at most 2^14 entries entering them, and the final fold,
    // in one CTA (form_tail_drawn_kernel)
    const int i0 = std::max(1, rounds - 13);
    for (int i = 1; i < i0; i++) {
      RoundArgs b{};
      for (int k = 0; k < nv; k++) {
        b.in[k] = i == 1 ? v[k] : buf[(i - 2) & 1][k];
        b.out[k] = buf[(i - 1) & 1][k];
      }
      b.pairs = n >> (i + 1);
      b.r = ch + (i - 1);
      b.partial = partial;
      form_step_launch(form, b, 1, round_blocks(b.pairs), s);
      k_sc_finish<<<1, kT, 0, s>>>(partial, round_blocks(b.pairs), nc, y, draw + first + (uint64_t)stride * i, ch, i,
                                   flags, bit, tr, op);
      check();
    }
    DrawnTailArgs t{};
    for (int k = 0; k < nv; k++) {
      t.in[k] = i0 == 1 ? v[k] : buf[(i0 - 2) & 1][k];
      t.buf[0][k] = buf[(i0 - 1) & 1][k];
      t.buf[1][k] = buf[i0 & 1][k];
    }
    t.n = n;
    t.i0 = i0;
    t.rounds = rounds;
    t.draw = draw;
    t.first = first;
    t.stride = stride;
    t.ch = ch;
    t.y = y;
    t.fin = fin;
    t.flags = flags;
    t.bit = bit;
    t.tr = tr;
    t.off_polys = op;
    t.off_fin = of;
    form_tail_drawn_launch(form, t, s);
  }

  // count F::_random() values, drawn ahead by the script
  fe *draws(int count) {
    if (script) script->push_back({DRAW_FIELDS, count, 0u, arena_used});
    fe *p = dry ? nullptr : arena + arena_used;
    arena_used += (uint64_t)count;
    return p;
  }
  // count rand() % mod values, drawn by the script into the transcript at off
  const int32_t *draw_mod(int count, uint32_t mod, uint64_t off) {
    if (script) script->push_back({DRAW_INTS, count, mod, off});
    return dry ? nullptr : reinterpret_cast<const int32_t *>(tr + off);
  }

  // The randomness the leader's delegation draws in one round:
  // prove_multi_folding log2 S + 1 + 5 rounds4 + 3 log2 d, then
  // prove_extension log2 S + 4 rounds3 + 1 + 3 log2 C0.
  struct RoundOut {
    fe *A = nullptr, *W = nullptr;  // the WHIR array (max_delegation) and its codeword
    fe *claim = nullptr;            // (value, point of log2 max_delegation)
    uint64_t off_root = 0;          // the root of its commitment in the transcript
  };

  RoundOut delegation_round(const LeaderRound &rd) {
    RoundOut out;
    const int l = rd.l, d = rd.d, logd = ilog2((uint64_t)d);
    uint64_t S = 1;
    while (S < (uint64_t)l) S <<= 1;
    const int logS = ilog2(S);
    const uint64_t md = in.max_delegation, Lw = 4 * md;
    const int logmd = ilog2(md);
    const uint64_t C0 = rd.C0;
    const int logC0 = ilog2(C0), lograte = ilog2(C0 / (uint64_t)d);
    if ((uint64_t)l * d > md) throw ArgError("pcs leader: segments exceed the delegation size");
    if (C0 > (1u << 13) || C0 < (uint64_t)d) throw ArgError("pcs leader: extension length out of range");
    if (d < 2 || d > 1024 || l > 1024) throw ArgError("pcs leader: degree or query count out of range");
    // Whir_Commit_initial(arr, 4, 8) of the gathered segments (coPCS.cpp:773-779):
    // the codeword and the root of MT_commit_Blake over it
    const uint64_t off_root = lay.rec(T_D_ROOT, 1, 32);
    out.off_root = off_root;
    out.A = alloc<fe>(md);
    out.W = alloc<fe>(Lw);
    if (!dry) {
      GBZ_CUDA(cudaMemsetAsync(out.A, 0, 16 * md, s));
      GBZ_CUDA(cudaMemcpyAsync(out.A, rd.seg, 16ull * l * d, cudaMemcpyDeviceToDevice, s));
      fe *tmp = alloc<fe>(Lw);
      ntt_launch(R.tables(ilog2(Lw)), out.A, (uint64_t)l * d, out.W, tmp, false, s);
      k_merkle_root<<<1, 32, 0, s>>>(out.W, ilog2(Lw / 4), tr, off_root);
      check();
    }
    // queries2[i] = rand() % C[0].size() (coPCS.cpp:789)
    const uint64_t off_q2 = lay.rec(T_D_QUERIES, (uint32_t)l, 4);
    const int32_t *q2 = draw_mod(l, (uint32_t)C0, off_q2);
    // ---- prove_multi_folding
    const int R4 = logS + logd;
    const int nd_pmf = logS + 1 + 5 * R4 + 3 * logd;
    const fe *D = draws(nd_pmf);
    fe *b1 = alloc<fe>(S), *twd = alloc<fe>(d), *y = alloc<fe>(1);
    fe *V[4];
    for (int k = 0; k < 4; k++) V[k] = alloc<fe>(S * d);
    const fe wn_inv = finv(root_of_unity(ilog2(rd.n)));
    if (!dry) {
      beta_launch(D, logS, b1, s);
      powers_launch(finv(root_of_unity(logd)), (uint64_t)d, twd, s);
      k_pmf_vectors<<<(unsigned)S, 256, 32ull * d, s>>>(rd.seg, rd.qpos, l, d, logd, twd, wn_inv, rd.L, b1, V[0],
                                                         V[1], V[2], V[3]);
      // K = d sum_t b1[t] y[t] (pad_vector(y): zeros beyond l)
      k_dot<<<1, kT, 0, s>>>(b1, rd.y, (uint64_t)l, fe_make((uint64_t)d, 0), y);
      check();
    }
    fe *ch4 = alloc<fe>(R4), *fin4 = alloc<fe>(4);
    {
      const fe *vv[4] = {V[0], V[1], V[2], V[3]};
      sumcheck(SC_QUADRUPLE, vv, S * d, y, D, logS + 1 + 4, 5, ch4, fin4, LF_ROUND);
    }
    fe *b12 = alloc<fe>(S), *b11 = alloc<fe>(d);
    if (!dry) {
      beta_launch(ch4 + logd, logS, b12, s);
      beta_launch(ch4, logd, b11, s);
      k_pmf_checks<<<1, kT, 0, s>>>(fin4, ch4, logd, logS, D, b12, b11, rd.L, rd.qpos, l, d, wn_inv, flags);
      check();
    }
    // the second sumcheck: sum_t b12[t] segment_t against the reduced matrix at r11
    fe *U1 = alloc<fe>(d), *U2 = alloc<fe>(d), *chq = alloc<fe>(logd), *finq = alloc<fe>(2);
    if (!dry) {
      k_seg_comb<<<d, kT, 0, s>>>(rd.seg, b12, l, d, U1);
      k_reduced_matrix<<<nblk(d), kT, 0, s>>>(ch4, logd, d, twd, U2);
      k_set<<<1, 32, 0, s>>>(y, fin4);
      check();
    }
    {
      const fe *vv[2] = {U1, U2};
      sumcheck(SC_QUADRATIC, vv, (uint64_t)d, y, D, logS + 1 + 5 * R4 + 2, 3, chq, finq, LF_DELEGATION);
    }
    // evaluate_vector scratch: halves of up to 2^13 entries
    fe *ev = alloc<fe>(1), *es = alloc<fe>(8192);
    if (!dry) {
      k_eval<<<1, kT, 0, s>>>(U2, logd, chq, es, es + 4096, ev);
      k_check_eq<<<1, 32, 0, s>>>(ev, finq + 1, flags, LF_DELEGATION);
      check();
    }
    // the claim (finq[0], r_q ++ r12) padded with zeros to log2 max_delegation
    const uint64_t off_claim = lay.rec(T_D_CLAIM, (uint32_t)(1 + logmd), 16);
    out.claim = alloc<fe>(1 + logmd);
    if (!dry) {
      k_claim<<<1, 64, 0, s>>>(finq, chq, logd, ch4 + logd, logS, logmd, out.claim, tr, off_claim);
      check();
    }
    // ---- extended segments and prove_extension
    const uint64_t off_o = lay.rec(T_D_OPEN, (uint32_t)l, 16);
    const int R3 = logS + logC0;
    const int nd_pe = logS + 4 * R3 + 1 + 3 * logC0;
    const fe *De = draws(nd_pe);
    fe *E = zeros(S * C0), *W2 = alloc<fe>(S * C0), *W3 = alloc<fe>(S * C0), *o = alloc<fe>(l), *bb = alloc<fe>(S);
    if (!dry) {
      ntt_batched(R.tables(logC0), rd.seg, (uint64_t)d, (uint32_t)d, E, (uint64_t)l, false, s);
      beta_launch(De, logS, bb, s);
      k_pe_vectors<<<nblk(S * C0), kT, 0, s>>>(E, q2, l, C0, bb, o, W2, W3, S * C0, tr, off_o);
      k_dot<<<1, kT, 0, s>>>(o, bb, (uint64_t)l, fe_one(), y);
      check();
    }
    fe *ch3 = alloc<fe>(R3), *fin3 = alloc<fe>(3);
    {
      const fe *vv[3] = {E, W2, W3};
      sumcheck(SC_CUBIC, vv, S * C0, y, De, logS + 3, 4, ch3, fin3, LF_ROUND);
    }
    fe *b1e = alloc<fe>(C0), *b2e = alloc<fe>(S);
    fe *v = zeros(C0), *Wp = alloc<fe>(C0), *chp = alloc<fe>(logC0), *finp = alloc<fe>(2);
    if (!dry) {
      beta_launch(ch3, logC0, b1e, s);
      beta_launch(ch3 + logC0, logS, b2e, s);
      k_pe_checks<<<1, kT, 0, s>>>(fin3, b1e, b2e, q2, l, ch3 + logC0, De, logS, flags);
      // prove_fft (delegate_protocol.cpp:119-145) of sum_t b2[t] segment_t at r1
      k_seg_comb<<<d, kT, 0, s>>>(rd.seg, b2e, l, d, v);
      const NttTables &tc = R.tables(logC0);
      k_phi<<<nblk(C0), kT, 0, s>>>(ch3, logC0, logC0, tc.lo_fwd, tc.hi_fwd, fe_one(), Wp);
      k_set<<<1, 32, 0, s>>>(y, fin3);
      check();
    }
    {
      const fe *vv[2] = {Wp, v};
      sumcheck(SC_QUADRATIC, vv, C0, y, De, logS + 4 * R3 + 1 + 2, 3, chp, finp, LF_DELEGATION);
    }
    const uint64_t off_ext = lay.rec(T_D_EXT_CLAIM, (uint32_t)(1 + logd + logS), 16);
    if (!dry) {
      k_eval<<<1, kT, 0, s>>>(Wp, logC0, chp, es, es + 4096, ev);
      k_check_eq<<<1, 32, 0, s>>>(ev, finp, flags, LF_DELEGATION);
      k_ext_claim<<<1, 32, 0, s>>>(finp, chp, logC0, lograte, ch3 + logC0, logS, tr, off_ext);
      check();
    }
    return out;
  }

  // The PIOP mode's WHIR batch slots 2 and 3 (coPCS.cpp:1620-1629): the
  // first two delegation rounds' arrays, codewords and roots, the betas of
  // their claims' points and the claims' values.
  void piop_slots(const std::vector<RoundOut> &ro) {
    if (ro.size() < 2) throw ArgError("pcs leader: the PIOP mode needs two delegation rounds");
    const uint64_t md = in.max_delegation;
    if (dry) return;
    for (int c = 0; c < 2; c++) {
      const WhirSlotDev &o = in.slot[c];
      if (o.arr) GBZ_CUDA(cudaMemcpyAsync(o.arr, ro[c].A, 16 * md, cudaMemcpyDeviceToDevice, s));
      if (o.cw) GBZ_CUDA(cudaMemcpyAsync(o.cw, ro[c].W, 64 * md, cudaMemcpyDeviceToDevice, s));
      if (o.betas) beta_launch(ro[c].claim + 1, ilog2(md), o.betas, s);
      if (o.claim) GBZ_CUDA(cudaMemcpyAsync(o.claim, ro[c].claim, 16, cudaMemcpyDeviceToDevice, s));
      if (o.root) GBZ_CUDA(cudaMemcpyAsync(o.root, tr + ro[c].off_root, 32, cudaMemcpyDeviceToDevice, s));
    }
  }

  // delegate_lagrange_eval(L1 = the input's Lagrange factors, L2 = the
  // rounds' Lagrange vectors, y = b2f, offset, _queries[0])
  // (delegate_protocol.cpp:603-710): the cubic sumcheck of (L2's tensor,
  // the transform of L1's tensor with its last q0 entries zeroed, omega^j)
  // and the checks of its three values, then the cubic sumcheck of (phi at
  // its point scaled by 1/Bs, L1's tensor, ones with the last q0 entries
  // zeroed) without round checks, L1's evaluation and the sum of the ones
  // vector.
  void lagrange_delegation(const fe *b2f, const fe *om) {
    const int nr = (int)in.rounds.size(), logBs = ilog2(in.Bs);
    const uint64_t Bs = in.Bs, q = in.q0;
    if (in.nlag < 1 || in.nlag > 8) throw ArgError("pcs leader: 1..8 Lagrange factors");
    int lsum = 0, lmax = 0;
    for (int k = 0; k < in.nlag; k++) {
      if (in.loglag[k] < 1 || in.loglag[k] > 30) throw ArgError("pcs leader: Lagrange factor length");
      lsum += in.loglag[k];
      lmax = std::max(lmax, in.loglag[k]);
    }
    if (lsum != logBs) throw ArgError("pcs leader: the Lagrange factors must multiply to the row length");
    if (q >= Bs) throw ArgError("pcs leader: _queries[0] must be below the row length");
    const uint64_t off_y = lay.rec(T_L_BETA_Y, 1, 16);
    const int nd = 2 * (1 + 4 * logBs);
    const fe *D = draws(nd);
    TensorArgs ta{}, t1{};
    ta.n = nr;
    for (int i = 0; i < nr; i++) {
      ta.L[i] = in.rounds[i].L;
      ta.logd[i] = ilog2((uint64_t)in.rounds[i].d);
    }
    t1.n = in.nlag;
    {
      uint64_t o = 0;
      for (int k = 0; k < in.nlag; k++) {
        t1.L[k] = in.lag ? in.lag + o : nullptr;
        t1.logd[k] = in.loglag[k];
        o += 1ull << in.loglag[k];
      }
    }
    fe *L2v = alloc<fe>(Bs), *L1v = alloc<fe>(Bs), *L1f = alloc<fe>(Bs), *ones = alloc<fe>(Bs), *y = alloc<fe>(1);
    if (!dry) {
      k_tensor<<<nblk(Bs), kT, 0, s>>>(ta, Bs, L2v);
      k_tensor<<<nblk(Bs), kT, 0, s>>>(t1, Bs, L1v);
      GBZ_CUDA(cudaMemcpyAsync(L1f, L1v, 16 * Bs, cudaMemcpyDeviceToDevice, s));
      if (q) GBZ_CUDA(cudaMemsetAsync(L1f + (Bs - q), 0, 16 * q, s));
      fe *tmp = alloc<fe>(Bs);
      ntt_launch(R.tables(logBs), L1f, Bs, L1f, tmp, false, s);
      k_fill_prefix<<<nblk(Bs), kT, 0, s>>>(ones, Bs, Bs - q);
      k_set<<<1, 32, 0, s>>>(y, b2f);
      k_put1<<<1, 32, 0, s>>>(b2f, tr, off_y);
      check();
    }
    fe *ch = alloc<fe>(logBs), *fin = alloc<fe>(3);
    {
      const fe *vv[3] = {L2v, L1f, om};
      sumcheck(SC_CUBIC, vv, Bs, y, D, 1 + 3, 4, ch, fin, LF_ROUND);
    }
    const uint64_t off_le = lay.rec(T_L_EVALS, (uint32_t)nr, 16);
    fe *W = alloc<fe>(Bs), *ch2 = alloc<fe>(logBs), *fin2 = alloc<fe>(3);
    if (!dry) {
      int dmax = 0;
      for (int i = 0; i < nr; i++) dmax = std::max(dmax, in.rounds[i].d);
      fe *es = alloc<fe>((uint64_t)std::max(dmax, 1 << lmax));
      k_beta_evals<<<1, kT, 0, s>>>(ta, ch, fin, LF_BETAS, es, flags, tr, off_le);
      k_lag_omega<<<1, 32, 0, s>>>(ch, logBs, root_of_unity(1 + in.log_rate_offset + logBs), fin, flags);
      const NttTables &tb = R.tables(logBs);
      k_phi<<<nblk(Bs), kT, 0, s>>>(ch, logBs, logBs, tb.lo_fwd, tb.hi_fwd, finv(fe_make(Bs, 0)), W);
      k_set<<<1, 32, 0, s>>>(y, fin + 1);
      check();
    }
    {
      const fe *vv[3] = {W, L1v, ones};
      sumcheck(SC_CUBIC, vv, Bs, y, D, (1 + 4 * logBs) + 1 + 3, 4, ch2, fin2, 0);
    }
    const uint64_t off_l1 = lay.rec(T_L_LAG_EVALS, (uint32_t)in.nlag, 16);
    if (!dry) {
      fe *es = alloc<fe>(1ull << lmax);
      k_beta_evals<<<1, kT, 0, s>>>(t1, ch2, fin2 + 1, LF_LAG2, es, flags, tr, off_l1);
      k_lag_ones<<<1, kT, 0, s>>>(fin2, ch2, logBs, Bs, q, flags);
      check();
    }
  }

  void run() {
    const int N = in.N, nr = (int)in.rounds.size();
    const uint64_t md = in.max_delegation, Lw = 4 * md;
    const int logmd = ilog2(md), logBs = ilog2(in.Bs);
    if (nr < 2 || nr > 8) throw ArgError("pcs leader: 2..8 rounds");
    if (in.n_final != 1) throw ArgError("pcs leader: the parties' final data must be one value each");
    std::vector<RoundOut> ro;
    for (int i = 1; i < nr; i++) ro.push_back(delegation_round(in.rounds[i]));
    const int nR = nr - 1;
    // decoding, unpack, final verification step 1
    const uint64_t off_unp = lay.rec(T_L_UNPACKED, (uint32_t)N, 16);
    fe *fp = alloc<fe>(N / 2), *fB = alloc<fe>(N / 2);
    if (!dry) {
      const uint64_t cpl = in.cpl_final;
      fe *dec = alloc<fe>((uint64_t)N * cpl);
      if (cpl >= 2) {
        fe *tmp = alloc<fe>((uint64_t)N * cpl);
        ntt_launch_rows(R.tables(ilog2(cpl)), in.Cp, cpl, cpl, dec, cpl, N, tmp, true, s);
      } else {
        GBZ_CUDA(cudaMemcpyAsync(dec, in.Cp, 16ull * N * cpl, cudaMemcpyDeviceToDevice, s));
      }
      k_decode_check<<<nblk((uint64_t)N * in.n_final), kT, 0, s>>>(dec, cpl, in.bcd, in.n_final, N, flags);
      k_unpack_final<<<1, 32, 0, s>>>(in.unpack, in.bcd, in.B, N, in.K, fp, fB, flags, tr, off_unp);
      check();
    }
    if (in.piop) {
      piop_slots(ro);
    } else {
      // aggregate_claims (Whir.cpp:608-668)
      const uint64_t off_ch = lay.rec(T_AGGR_CHALLENGES, (uint32_t)(2 * nR), 16), off_K = lay.rec(T_AGGR_K, 1, 16);
      fe *betas[8] = {}, *sums = alloc<fe>((uint64_t)nR * nR);
      fe *arr = alloc<fe>(md), *baggr = alloc<fe>(md), *cw = alloc<fe>(Lw);
      for (int c = 0; c < nR; c++) betas[c] = alloc<fe>(md);
      if (!dry) {
        for (int c = 0; c < nR; c++) beta_launch(ro[c].claim + 1, logmd, betas[c], s);
        VecList va{}, vb{};
        for (int i = 0; i < nR; i++) {
          va.p[i] = ro[i].A;
          vb.p[i] = betas[i];
        }
        fe *mdp = alloc<fe>(multidot_scratch(md));
        multidot_launch(va, nR, vb, nR, md, mdp, sums, s);
      }
      const fe *ch = draws(2 * nR);
      if (!dry) {
        k_aggr_K<<<1, 32, 0, s>>>(sums, ch, nR, st, tr, off_ch, off_K);
        check();
        VecList va{}, vb{}, vc{};
        for (int i = 0; i < nR; i++) {
          va.p[i] = ro[i].A;
          vb.p[i] = betas[i];
          vc.p[i] = ro[i].W;
        }
        lincomb_launch(vb, ch, nR, md, baggr, false, s);
        lincomb_launch(va, ch + nR, nR, md, arr, false, s);
        // aggregate_commitments (Whir.cpp:547-606): the codeword, the openings
        // in the first commitment, the tree over zero leaves (whir_k = 8)
        lincomb_launch(vc, ch + nR, nR, Lw, cw, false, s);
      }
      const int la = whir_query_count(4), depth_a = ilog2(Lw / 4);
      const uint64_t off_aq = lay.rec(T_AGGR_QUERIES, (uint32_t)la, 4);
      const uint64_t off_ap = lay.rec(T_AGGR_PATHS, (uint32_t)(la * depth_a), 32);
      const uint64_t off_ar = lay.rec(T_AGGR_ROOT, 1, 32);
      draw_mod(la, (uint32_t)(Lw / 4), off_aq);
      if (!dry) {
        k_whir_paths_chain<<<nblk((uint64_t)la * depth_a, 128), 128, 0, s>>>(ro[0].W, Lw / 4, la, tr, off_aq, off_ap,
                                                                             0, 0);
        k_zero_tree_root<<<1, 32, 0, s>>>(ilog2(Lw / 8), tr, off_ar);
        check();
      }
      // _Whir_Open (Whir.cpp:469-545) with whir_k = 8 from the zero-leaf tree
      const uint64_t sizes[1] = {md};
      const BatchPlan P = batch_plan(1, sizes, 4, 8, Lw / 8);
      BatchResources br;
      br.s = s;
      br.buf = [this](int slot, uint64_t bytes) -> void * {
        auto it = slots.find(slot);
        if (it != slots.end()) return it->second;
        void *p = R.alloc(bytes);
        slots[slot] = p;
        return p;
      };
      br.tables = R.tables;
      br.st = st;
      br.ub_scratch = alloc<fe>(kUpdateBetasScratch);
      WalkTrace wt;
      // the opening draws from st->prng itself: the script leaves its state
      // there and skips the opening's calls (per iteration log2 kappa
      // F::_random(), the queries' rand(), update_betas' F::_random(); the
      // final point's F::_random())
      if (script) script->push_back({DRAW_STATE, 0, 0u, 0});
      {
        const fe *arrays[1] = {arr}, *bets[1] = {baggr}, *cws[1] = {cw};
        batch_open_walk(br, P, arrays, bets, cws, nullptr, tr, lay, dry, &wt);
      }
      {
        uint64_t calls = 0;
        for (const BatchStep &e : P.steps)
          if (e.iterate) calls += 40ull * ilog2((uint64_t)e.kappa) + (uint64_t)e.l + 40;
        calls += 40ull * ilog2(P.m_final);
        if (script) script->push_back({DRAW_SKIP, (int)calls, 0u, 0});
        if (!dry) {
          k_prng_check<<<1, 32, 0, s>>>(st, after_walk, flags);
          check();
        }
      }
      const int npt = (int)wt.chal.size() + ilog2(wt.m_final);
      if (npt != logmd || (int)wt.chal.size() > 64 || (int)wt.queries.size() > kMaxTailIter)
        throw ArgError("pcs leader: WHIR opening shape");
      const uint64_t off_wc = lay.rec(T_L_WHIR_CLAIM, (uint32_t)(1 + logmd), 16);
      if (!dry) {
        const NttTables &tf = R.tables(ilog2(wt.L_final));
        k_reencode_check<<<nblk(wt.L_final), kT, 0, s>>>(wt.final_arr, (int)wt.m_final, wt.last_codeword, wt.L_final,
                                                        tf.lo_fwd, tf.hi_fwd, st);
        k_whir_flags<<<1, 32, 0, s>>>(st, flags);
        // the final claim (evaluate_vector(_initial_b, total_r), total_r)
        ChalOffs co{};
        co.n = (int)wt.chal.size();
        for (int i = 0; i < co.n; i++) co.off[i] = wt.chal[i];
        fe *total_r = alloc<fe>(logmd), *eb = alloc<fe>(md), *val = alloc<fe>(1), *mdp = alloc<fe>(multidot_scratch(md));
        k_gather_r<<<1, 64, 0, s>>>(tr, co, wt.final_point, ilog2(wt.m_final), total_r);
        beta_launch(total_r, logmd, eb, s);
        VecList a1{}, a2{};
        a1.p[0] = eb;
        a2.p[0] = baggr;
        multidot_launch(a1, 1, a2, 1, md, mdp, val, s);
        k_put_claim_value<<<1, 64, 0, s>>>(val, total_r, logmd, tr, off_wc);
        check();
        // verification step 3
        Step3Args a3{};
        a3.iters = (int)wt.queries.size();
        a3.nr = logmd;
        int skip = 0;
        for (int i = 0; i < a3.iters; i++) {
          skip += ilog2((uint64_t)wt.kappa[i]);
          a3.off_q[i] = wt.queries[i];
          a3.off_c[i] = wt.comb[i];
          a3.NL[i] = wt.NL[i];
          a3.l[i] = wt.l[i];
          a3.skip[i] = skip;
        }
        a3.R = nR;
        a3.npt = logmd;
        a3.off_eval = wt.final_eval;
        a3.off_claim = off_wc;
        fe *claims = alloc<fe>((uint64_t)nR * (1 + logmd));
        for (int c = 0; c < nR; c++)
          GBZ_CUDA(cudaMemcpyAsync(claims + (uint64_t)c * (1 + logmd), ro[c].claim, 16ull * (1 + logmd),
                                   cudaMemcpyDeviceToDevice, s));
        k_whir_step3<<<1, kT, 0, s>>>(tr, a3, claims, ch, total_r, flags);
        check();
      }
    }
    // r_c and the final verification step
    const uint64_t off_rc = lay.rec(T_L_RC, 2, 16);
    const fe *rc = draws(1);
    // the leader's b2: omega^j times the transform of beta(r2), folded by every round's L
    const fe om_off = root_of_unity(1 + in.log_rate_offset + logBs);
    fe *om = alloc<fe>(in.Bs), *b2c = alloc<fe>(in.Bs), *b2t = alloc<fe>(in.Bs), *b2f = nullptr;
    if (!dry) {
      powers_launch(om_off, in.Bs, om, s);
      k_mul<<<nblk(in.Bs), kT, 0, s>>>(in.b2, om, in.Bs, b2c);
      check();
      fe *cur = b2c, *nxt = b2t;
      uint64_t len = in.Bs;
      for (int i = 0; i < nr; i++) {
        const int lg = ilog2((uint64_t)in.rounds[i].d);
        cophase2_launch(cur, len, in.rounds[i].L, lg, nxt, s);
        len >>= lg;
        std::swap(cur, nxt);
      }
      if (len != 1) throw ArgError("pcs leader: the fold degrees do not multiply to the row length");
      b2f = cur;
      FinalArgs fa{};
      fa.N = N;
      fa.nq = nr - 1;
      uint64_t rows = in.Bs;  // instance_size[i + 2] = Bs / (d_0 ... d_i)
      for (int j = 0; j < nr - 1; j++) {
        const LeaderRound &q = in.rounds[j];
        FinalRound &f = fa.q[j];
        rows /= (uint64_t)q.d;
        f.s = q.s;
        f.qp = q.qp;
        f.qpos = q.qpos;
        f.l = q.l;
        f.mul = q.rate_next;
        f.div = q.rate_cur;
        f.nL = nr - 1 - j;
        for (int k = 0; k < f.nL; k++) {
          f.L[k] = in.rounds[j + 1 + k].L;
          f.d[k] = in.rounds[j + 1 + k].d;
        }
        f.rows = rows;
        f.rate = in.rate0[j + 2];
      }
      fa.fB = fB;
      fa.b3 = in.b3;
      fa.r_first = in.r_first;
      fa.b2f = b2f;
      fa.rc = rc;
      fa.off_rc = off_rc;
      int nterms = 0;
      for (int j = 0; j < fa.nq; j++) nterms += fa.q[j].l;
      fe *py = alloc<fe>(64), *terms = alloc<fe>(std::max(nterms, 1));
      k_powers_y<<<1, 64, 0, s>>>(N, rc, py);
      if (nterms) k_final_terms<<<nblk((uint64_t)nterms * 32), kT, 0, s>>>(fa, py, terms);
      k_final_eval<<<1, kT, 0, s>>>(fa, terms, nterms, flags, tr);
      check();
    }
    if (in.piop) {
      lagrange_delegation(b2f, om);
      return;
    }
    // delegate_beta_eval(r2, Lagrange_Evals, b2[0], offset)
    const uint64_t off_by = lay.rec(T_L_BETA_Y, 1, 16);
    const int nd_b = 1 + 4 * logBs + 1 + 3 * (logBs + 1);
    const fe *Db = draws(nd_b);
    TensorArgs ta{};
    ta.n = nr;
    for (int i = 0; i < nr; i++) {
      ta.L[i] = in.rounds[i].L;
      ta.logd[i] = ilog2((uint64_t)in.rounds[i].d);
    }
    fe *Lv = alloc<fe>(in.Bs), *y = alloc<fe>(1);
    if (!dry) {
      k_tensor<<<nblk(in.Bs), kT, 0, s>>>(ta, in.Bs, Lv);
      k_set<<<1, 32, 0, s>>>(y, b2f);
      k_put1<<<1, 32, 0, s>>>(b2f, tr, off_by);
      check();
    }
    fe *chb = alloc<fe>(logBs), *finb = alloc<fe>(3);
    {
      const fe *vv[3] = {Lv, in.b2, om};
      sumcheck(SC_CUBIC, vv, in.Bs, y, Db, 1 + 3, 4, chb, finb, LF_ROUND);
    }
    const uint64_t off_le = lay.rec(T_L_EVALS, (uint32_t)nr, 16);
    fe *Wr = alloc<fe>(2 * in.Bs), *bx = zeros(2 * in.Bs), *chw = alloc<fe>(logBs + 1), *finw = alloc<fe>(2);
    if (!dry) {
      fe *es = alloc<fe>(1024);
      k_beta_evals<<<1, kT, 0, s>>>(ta, chb, finb, LF_BETAS, es, flags, tr, off_le);
      const NttTables &t2 = R.tables(logBs + 1);
      k_phi<<<nblk(2 * in.Bs), kT, 0, s>>>(chb, logBs, logBs + 1, t2.lo_fwd, t2.hi_fwd, fe_one(), Wr);
      // b = precompute_beta(r2), zero beyond its length (the reference reads
      // past the end of b there: the value is never used)
      beta_launch(in.r2, logBs, bx, s);
      k_set<<<1, 32, 0, s>>>(y, finb + 1);
      check();
    }
    {
      const fe *vv[2] = {Wr, bx};
      sumcheck(SC_QUADRATIC, vv, 2 * in.Bs, y, Db, 1 + 4 * logBs + 1 + 2, 3, chw, finw, 0);
    }
  }
};

}  // namespace

void leader_tail(LeaderResources &R, const LeaderInputs &in, ProofState *st, uint32_t *flags, uint8_t *tr,
                 Layout &lay, std::vector<DrawOp> *script, uint64_t *arena_len, const LeaderDraws *draws) {
  Tail t{R, in, st, flags, tr, lay, tr == nullptr, R.s, script, draws ? draws->after_walk : nullptr,
         draws ? draws->arena : nullptr, 0, {}};
  t.run();
  if (arena_len) *arena_len = t.arena_used;
}

void leader_tail_init(ProofState *st, const glibc_prng &g, uint32_t *flags, cudaStream_t s) {
  k_tail_init<<<1, 32, 0, s>>>(st, g, flags);
  GBZ_CUDA(cudaGetLastError());
}

void leader_draws_launch(const glibc_prng &g0, const DrawOp *ops, int nops, const LeaderDraws &d, uint8_t *tr,
                         ProofState *st, cudaStream_t s) {
  k_draw_script<<<1, 32, 0, s>>>(g0, ops, nops, d.arena, tr, st, d.after_walk, d.final_state);
  GBZ_CUDA(cudaGetLastError());
}

}  // namespace gbz
