// The collaborative PCS of N parties on one device: PCS_commit and the
// parties' side of PCS_open_new with the leader's aggregation of their round
// messages (coPCS.cpp:236-250, 1310-1607), as the reference runs them with
// one MPI rank per party.
//
// PcsLayout: every per-party vector is one party-major device array
// [party][entry]; a step that every rank runs on its own share is one launch
// over all parties (grid.y = party) or one batched transform over the
// concatenated rows.  The leader's work (unpacking the packed-Shamir round
// messages, Fiat-Shamir challenges, the query draws and the running claim)
// runs on the device too, in one-CTA kernels, so an opening is a stream of
// launches with no host round trip.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gbz_copcs.cuh"
#include "gbz_ctx.cuh"
#include "gbz_pcs_leader.cuh"

using namespace gbz_api;

namespace gbz {
namespace {

constexpr int kPcsMaxParties = 64;     // packed Shamir with N / 2 <= 32 values per group
constexpr int kPcsMaxQueries = 1024;   // queries of one delegate check
constexpr int kPcsMaxRounds = 8;       // rates.size()
constexpr int kPcsMaxLogDeg = 10;      // the block fold of phase 2 (d <= 1024)

// Transcript tags of the opening (see include/gbz.h).
enum : uint32_t {
  T_PCS_ROOTS = 32, T_PCS_LEADER_ROOT = 33, T_PCS_PARTY_POLYS = 34, T_PCS_POLY = 35, T_PCS_CHALLENGE = 36,
  T_PCS_QUERIES = 37, T_PCS_Y = 38, T_PCS_SEGMENTS = 39, T_PCS_S = 40, T_PCS_K = 41, T_PCS_FINAL = 42,
  T_COSC_FINAL_SHARES = 43, T_COSC_UNPACKED = 44, T_COSC_CLAIMS = 45
};

// Verifier-side state of one opening, resident on the device.
struct PcsDev {
  fe fs;         // Fiat-Shamir chain (prev_challenge, Fiat_Shamir.cpp:5)
  fe K;          // running claim
  fe r_first;    // challenge of the batching round
  fe c;          // challenge of the current round
  fe s;          // phase-3 challenge of the current round
  uint32_t error;  // bit 0: a round message does not match K; bit 1: a delegate check failed
};

__device__ __forceinline__ fe pow_tab(const fe *lo, const fe *hi, uint64_t e) {
  return fmul(lo[e & 4095u], hi[e >> 12]);
}

__device__ __forceinline__ void put_hash(uint8_t *tr, uint64_t off, const uint32_t h[8]) {
  uint32_t *p = reinterpret_cast<uint32_t *>(tr + off);
  for (int k = 0; k < 8; k++) p[k] = h[k];
}

// G(h) = blake3(h || h): an inner node of create_tree_blake whose left child
// is h (merkle_tree.cpp:267-299 hashes the left child twice).
__device__ void self_hash(uint32_t h[8], int times) {
  uint32_t m[16];
  for (int t = 0; t < times; t++) {
    for (int k = 0; k < 8; k++) m[k] = m[8 + k] = h[k];
    blake3_block64(m, h);
  }
}

// Record headers {tag, count} at their offsets (built by the host).
struct Hdr {
  uint64_t off;
  uint32_t tag, count;
};
__global__ void k_headers(const Hdr *h, int n, uint8_t *tr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t *p = reinterpret_cast<uint32_t *>(tr + h[i].off);
  p[0] = h[i].tag;
  p[1] = h[i].count;
}

__global__ void k_init(PcsDev *st, fe fs, fe K) {
  st->fs = fs;
  st->K = K;
  st->r_first = st->c = st->s = fe_zero();
  st->error = 0;
}

// b3' = the packed-Shamir share map applied to b3 (coPCS.cpp:1370-1376):
// party j's scale of the beta vector.
__global__ void k_b3p(const fe *b3, int nb3, const fe *mu, int N, fe *b3p) {
  const int j = threadIdx.x;
  if (j >= N) return;
  fe acc = fe_zero();
  for (int t = 0; t < nb3; t++) acc = fadd(acc, fmul(mu[j * (N / 2) + t], b3[t]));
  b3p[j] = acc;
}

// out[p][j] = sum_{i < nrows} coef[i] rows[p][i][j] (coPCS.cpp:1352-1356).
__global__ void k_lincomb(const fe *rows, uint64_t pstride, uint64_t rstride, int nrows, uint64_t len, const fe *coef,
                          fe *out, uint64_t ostride) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= len) return;
  const fe *r = rows + blockIdx.y * pstride + j;
  fe acc = fe_zero();
  for (int i = 0; i < nrows; i++) acc = fadd(acc, fmul(coef[i], r[(uint64_t)i * rstride]));
  out[blockIdx.y * ostride + j] = acc;
}

// After the inverse transforms: bcd, cdl *= omega^{-j}; B = b2 omega^j b3'[p]
// (coPCS.cpp:1385-1397), omega = w_{2 rate_offset Bs}.
__global__ void k_open_prep(fe *bcd, fe *cdl, fe *B, const fe *b2, const fe *b3p, uint64_t Bs, const fe *lo,
                            const fe *hi, const fe *ilo, const fe *ihi) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= Bs) return;
  const uint64_t at = blockIdx.y * Bs + j;
  const fe wi = pow_tab(ilo, ihi, j);
  bcd[at] = fmul(bcd[at], wi);
  cdl[at] = fmul(cdl[at], wi);
  B[at] = fmul(fmul(b2[j], pow_tab(lo, hi, j)), b3p[blockIdx.y]);
}

// First batching round (coPCS.cpp:1403-1410): per party
// (sum (bcd - cdl) B, sum cdl B, 0), as per-CTA partials.
constexpr int kRedThreads = 256;
__global__ void __launch_bounds__(kRedThreads)
k_first_partial(const fe *bcd, const fe *cdl, const fe *B, uint64_t Bs, fe *partial) {
  __shared__ fe ra[kRedThreads], rb[kRedThreads];
  const uint64_t base = blockIdx.y * Bs;
  fe a = fe_zero(), b = fe_zero();
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < Bs; j += (uint64_t)gridDim.x * blockDim.x) {
    const fe x = bcd[base + j], y = cdl[base + j], w = B[base + j];
    a = fadd(a, fmul(fsub(x, y), w));
    b = fadd(b, fmul(y, w));
  }
  ra[threadIdx.x] = a;
  rb[threadIdx.x] = b;
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      ra[threadIdx.x] = fadd(ra[threadIdx.x], ra[threadIdx.x + s]);
      rb[threadIdx.x] = fadd(rb[threadIdx.x], rb[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    fe *o = partial + 2 * ((uint64_t)blockIdx.y * gridDim.x + blockIdx.x);
    o[0] = ra[0];
    o[1] = rb[0];
  }
}

// Party messages H[p] = (a, b, 0) from the partials; also their record.
__global__ void k_first_reduce(const fe *partial, int nblk, int N, fe *H, uint8_t *tr, uint64_t off_pp) {
  const int p = threadIdx.x;
  if (p >= N) return;
  fe a = fe_zero(), b = fe_zero();
  for (int k = 0; k < nblk; k++) {
    a = fadd(a, partial[2 * ((uint64_t)p * nblk + k)]);
    b = fadd(b, partial[2 * ((uint64_t)p * nblk + k) + 1]);
  }
  H[3 * p] = a;
  H[3 * p + 1] = b;
  H[3 * p + 2] = fe_zero();
  put_fe(tr, off_pp + 48ull * p, a);
  put_fe(tr, off_pp + 48ull * p + 16, b);
  put_fe(tr, off_pp + 48ull * p + 32, fe_zero());
}

// The leader's check and challenge of the batching round (coPCS.cpp:1428-1435).
__global__ void k_first_verify(PcsDev *st, const fe *poly, uint8_t *tr, uint64_t off_poly, uint64_t off_chal,
                               uint64_t off_K) {
  if (threadIdx.x) return;
  const fe p0 = poly[0], p1 = poly[1], p2 = poly[2];
  if (!fe_eq(fadd(p0, p1), st->K)) st->error |= 1;
  fe fs = st->fs;
  fs = hash_F(fs, p0);
  fs = hash_F(fs, p1);
  fs = hash_F(fs, p2);
  st->fs = fs;
  st->r_first = fs;
  st->K = fmul(fs, fadd(p1, fmul(fs, p0)));
  put_fe(tr, off_poly, p0);
  put_fe(tr, off_poly + 16, p1);
  put_fe(tr, off_poly + 32, p2);
  put_fe(tr, off_chal, fs);
  put_fe(tr, off_K, st->K);
}

// The fold of the batching round (coPCS.cpp:1438-1447): B *= r,
// bcd = r bcd + (1 - r) cdl, C' = r C' + (1 - r) codeword[batches - 1].
__global__ void k_first_fold(fe *bcd, const fe *cdl, fe *B, fe *Cp, const fe *cw_last, uint64_t cw_pstride,
                             uint64_t Bs, uint64_t L, const PcsDev *st) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= L) return;
  const fe r = st->r_first, om = fsub(fe_one(), r);
  const uint64_t p = blockIdx.y;
  Cp[p * L + j] = fadd(fmul(r, Cp[p * L + j]), fmul(om, cw_last[p * cw_pstride + j]));
  if (j < Bs) {
    const uint64_t at = p * Bs + j;
    B[at] = fmul(r, B[at]);
    bcd[at] = fadd(fmul(r, bcd[at]), fmul(om, cdl[at]));
  }
}

// Commitment roots of every party and the leader's root.  A party's root
// of MT_commit_Blake over a vector depends on its first leaf only: the
// leaf hash of entries e_k = data[p pstride + k estride] (k < 4), hashed
// `levels` more times (inner nodes hash their left child twice).  With
// `stale`, the parties report those roots instead (commit_tensorcode on a
// reused, deeper tree; see the host side).  The leader's root over N party
// roots is party 0's root hashed log2(N) times.
__global__ void k_roots(const fe *data, uint64_t pstride, uint64_t estride, int levels, int N, int logN,
                        const uint8_t *stale, uint8_t *roots, uint8_t *tr, uint64_t off_roots, uint64_t off_leader) {
  __shared__ uint32_t r0[8];
  const int p = threadIdx.x;
  if (p < N) {
    uint32_t h[8];
    if (stale) {
      for (int k = 0; k < 8; k++) h[k] = reinterpret_cast<const uint32_t *>(stale + 32 * p)[k];
    } else {
      const fe *d = data + (uint64_t)p * pstride;
      uint32_t m[16];
      fe4_words(d[0], d[estride], d[2 * estride], d[3 * estride], m);
      blake3_block64(m, h);
      self_hash(h, levels);
    }
    for (int k = 0; k < 8; k++) reinterpret_cast<uint32_t *>(roots + 32 * p)[k] = h[k];
    put_hash(tr, off_roots + 32ull * p, h);
    if (p == 0)
      for (int k = 0; k < 8; k++) r0[k] = h[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t h[8];
    for (int k = 0; k < 8; k++) h[k] = r0[k];
    self_hash(h, logN);
    put_hash(tr, off_leader, h);
  }
}

// get_indexes (Fiat_Shamir.cpp:37-56) for every party at once: l draws of
// (party, position) from the chain, then the order the leader holds them in
// after get_segments (MPI_utils.cpp:187-255): party 0's queries, then party
// 1's, ..., each in draw order.
__global__ void k_indexes(PcsDev *st, int l, int N, uint32_t Mq, int32_t *qp, int32_t *qpos, uint8_t *tr,
                          uint64_t off) {
  __shared__ int32_t sp[kPcsMaxQueries], sq[kPcsMaxQueries];
  __shared__ int32_t start[kPcsMaxParties + 1];
  if (threadIdx.x == 0) {
    // N and Mq are powers of two (checked by the host): % is a mask
    fe fs = st->fs;
    for (int i = 0; i < l; i++) {
      fs = hash_F(fs, fs);
      sp[i] = (int32_t)(fs.re & (uint64_t)(N - 1));
      sq[i] = (int32_t)(fs.im & (uint64_t)(Mq - 1));
    }
    st->fs = fs;
    for (int p = 0; p <= N; p++) start[p] = 0;
    for (int i = 0; i < l; i++) start[sp[i] + 1]++;
    for (int p = 0; p < N; p++) start[p + 1] += start[p];
    for (int i = 0; i < l; i++) {
      const int at = start[sp[i]]++;
      qp[at] = sp[i];
      qpos[at] = sq[i];
    }
  }
  __syncthreads();
  uint32_t *w = reinterpret_cast<uint32_t *>(tr + off);
  for (int i = threadIdx.x; i < l; i += blockDim.x) {
    w[2 * i] = (uint32_t)qp[i];
    w[2 * i + 1] = (uint32_t)qpos[i];
  }
}

// The leader's check of round i and its challenge (coPCS.cpp:1463-1483):
// sum_j poly[2j] = K, c = hash_to_field(poly), K = sum_k poly[k] L2[k] with
// L2 = compute_lagrange_coeff(c, 2d), and the fold weights L = the same at
// length d (utils.cpp:169-197: the inverse transform of the powers of c).
// scratch: 2 * 2d entries.
__global__ void __launch_bounds__(256)
k_round_verify(PcsDev *st, const fe *poly, int logd, fe wi, fe invD, fe invd, fe *L, fe *scratch, uint8_t *tr,
               uint64_t off_poly, uint64_t off_chal) {
  __shared__ fe red[256];
  __shared__ fe chal;
  __shared__ fe sh_cw[2 * 1024];  // the powers of c and of w^-1 (global scratch beyond 1024 points)
  const int d = 1 << logd, D = 2 * d;
  fe *cp = D <= 1024 ? sh_cw : scratch, *wp = D <= 1024 ? sh_cw + D : scratch + D;
  // (wi = omega_D^-1, invD, invd: constants of the shape, formed on the host)
  for (int k = threadIdx.x; k < D; k += blockDim.x) {
    wp[k] = fpow(wi, (uint64_t)k);
    put_fe(tr, off_poly + 16ull * k, poly[k]);
  }
  if (threadIdx.x == 0) {
    fe ev = fe_zero();
    for (int j = 0; j < d; j++) ev = fadd(ev, poly[2 * j]);
    if (!fe_eq(ev, st->K)) st->error |= 1;
    fe fs = st->fs;
    for (int k = 0; k < D; k++) fs = hash_F(fs, poly[k]);
    st->fs = fs;
    st->c = fs;
    put_fe(tr, off_chal, fs);
    chal = fs;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < D; k += blockDim.x) cp[k] = fpow(chal, (uint64_t)k);
  __syncthreads();
  // L2[k] = (1/D) sum_j c^j w^{-jk}; K' = sum_k poly[k] L2[k]
  fe acc = fe_zero();
  for (int k = threadIdx.x; k < D; k += blockDim.x) {
    fe s = fe_zero();
    for (int j = 0; j < D; j++) s = fadd(s, fmul(cp[j], wp[((uint64_t)j * k) & (D - 1)]));
    acc = fadd(acc, fmul(poly[k], fmul(s, invD)));
  }
  // L[k] = (1/d) sum_{j<d} c^j w_d^{-jk}, w_d^{-1} = (w_D^{-1})^2
  for (int k = threadIdx.x; k < d; k += blockDim.x) {
    fe s = fe_zero();
    for (int j = 0; j < d; j++) s = fadd(s, fmul(cp[j], wp[(2ull * j * k) & (D - 1)]));
    L[k] = fmul(s, invd);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fadd(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) st->K = red[0];
}

// delegate_checks (coPCS.cpp:753-763): per query j (party a, position q),
// the segment C'_a[q + k seg_n] (k < d) and its RS fold y_j (RS_multifold_segment
// equals output q of RS_multifold5 over C'_a).
__global__ void k_gather(const fe *Cp, uint64_t pstride, uint64_t seg_n, int d, const fe *fold, uint64_t fstride,
                         const int32_t *qp, const int32_t *qpos, int l, fe *y, uint8_t *tr, uint64_t off_y,
                         uint64_t off_seg, fe *seg_out) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint64_t)l * d) return;
  const int j = (int)(t / d), k = (int)(t % d);
  const uint64_t a = (uint64_t)qp[j], q = (uint64_t)qpos[j];
  const fe v = Cp[a * pstride + q + k * seg_n];
  put_fe(tr, off_seg + 16 * t, v);
  if (seg_out) seg_out[t] = v;
  if (k == 0) {
    const fe v = fold[a * fstride + q];
    y[j] = v;
    put_fe(tr, off_y + 16ull * j, v);
  }
}

// The check of coPCS.cpp:1521-1529: the new codeword holds y_j at the
// query's position scaled by rate_{i+2} / rate_{i+1}.
__global__ void k_check_y(const fe *Cpn, uint64_t pstride, uint32_t mul, uint32_t div, const int32_t *qp,
                          const int32_t *qpos, const fe *y, int l, PcsDev *st) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= l) return;
  const uint64_t pos = (uint64_t)mul * (uint32_t)qpos[j] / div;
  if (pos >= pstride || !fe_eq(Cpn[(uint64_t)qp[j] * pstride + pos], y[j])) atomicOr(&st->error, 2u);
}

// s = hash_to_field({0}) and, unless the last round, K += sum_j s^{j+1} y_j
// (coPCS.cpp:1535-1547).
// K += sum_j s^(j+1) y_j: term j on thread j mod 256 (s^(j+1) by
// squarings), the block's sum on thread 0.  Launched with 256 threads.
__global__ void __launch_bounds__(256)
k_s_update(PcsDev *st, const fe *y, int l, int addK, uint8_t *tr, uint64_t off_s, uint64_t off_K) {
  __shared__ fe sh_s;
  __shared__ fe red[256];
  if (threadIdx.x == 0) {
    sh_s = hash_F(st->fs, fe_zero());
    st->fs = sh_s;
    st->s = sh_s;
  }
  __syncthreads();
  const fe s = sh_s;
  fe acc = fe_zero();
  if (addK)
    for (int j = threadIdx.x; j < l; j += blockDim.x) acc = fadd(acc, fmul(fpow(s, (uint64_t)j + 1), y[j]));
  red[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x) return;
  fe K = st->K;
  for (int t = 0; t < (int)blockDim.x; t++) K = fadd(K, red[t]);
  st->K = K;
  put_fe(tr, off_s, s);
  put_fe(tr, off_K, K);
}

// pcs_sumcheck_phase3 (coPCS.cpp:634-648) for every party: B_p[j] +=
// sum_i s^{i+1} scale(a_i, p) (w^{q_i})^j, w = w_W, W = rate rows, q_i the
// query position scaled as the reference scales it, scale(a, p) the tensor
// scale of tensor_eval_vector (coPCS.cpp:610-632; a constant table).  For
// j < rows that is the forward transform of length W of the sparse vector
// V_p[q_i] += s^{i+1} scale(a_i, p): the prep writes q_i and the weights,
// the scatter sums the weights of equal positions (the first query at a
// position writes it), one batched transform over the N rows follows.
__global__ void k_phase3_prep(const PcsDev *st, const int32_t *qp, const int32_t *qpos, int l, uint32_t mul,
                              uint32_t div, int logw, const fe *scale, int N, uint32_t *q, fe *w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= l) return;
  q[i] = (uint32_t)(((uint64_t)mul * (uint32_t)qpos[i] / div) & ((1ull << logw) - 1));
  const fe si = fpow(st->s, (uint64_t)i + 1);
  for (int p = 0; p < N; p++) w[(uint64_t)p * l + i] = fmul(si, scale[qp[i] * N + p]);
}

// V (N x W, zero) gets V[p][q_i] = sum of w[p][j] over the queries j at q_i.
__global__ void k_phase3_scatter(const uint32_t *q, const fe *w, int l, uint64_t W, fe *V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= l) return;
  const uint64_t p = blockIdx.y;
  const uint32_t qi = q[i];
  for (int j = 0; j < i; j++)
    if (q[j] == qi) return;
  const fe *wp = w + p * l;
  fe acc = wp[i];
  for (int j = i + 1; j < l; j++)
    if (q[j] == qi) acc = fadd(acc, wp[j]);
  V[p * W + qi] = acc;
}

// B[p][j] += T[p][j] for j < rows (T: N rows of W entries).
__global__ void k_phase3_add(fe *B, uint64_t rows, const fe *T, uint64_t W) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= rows) return;
  const uint64_t p = blockIdx.y;
  B[p * rows + j] = fadd(B[p * rows + j], T[p * W + j]);
}

// The RS fold of a codeword by d (RS_multifold5, coPCS_utils.cpp:386-437, and
// RS_multifold_segment, :172-232) for any d: its butterflies compute, for
// output i, d f_c(x^d) (c < d, f(X) = sum_c X^c f_c(X^d), x = w_n^i) and
// return sum_c L[c] f_c(x^d).  With s_t = cw[i + t m] = f(x w_d^t) (m = n/d)
// that is (1/d) sum_t s_t P_L(w_n^{-(i + t m)}), P_L(z) = sum_c L[c] z^c, and
// Q[e] = P_L(w_n^{-e}) = n IDFT_n(L, zero-padded)[e].  So
// out[p][i] = (n/d) sum_t cw[p][i + t m] iQ[i + t m],  iQ = IDFT_n(L padded).
__global__ void k_fold_q(const fe *cw, uint64_t n, int logd, const fe *iQ, fe scale, fe *out, uint64_t ostride) {
  const uint64_t m = n >> logd;
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const fe *c = cw + blockIdx.y * n;
  fe acc = fe_zero();
  for (int t = 0; t < (1 << logd); t++) acc = fadd(acc, fmul(c[i + t * m], iQ[i + t * m]));
  out[blockIdx.y * ostride + i] = fmul(acc, scale);
}

// F_ip's local inner product (MPI_utils.cpp:489-491) of every party:
// sum_{i < nrows} sum_j rows[p][i][j] v1[32 j + i] (v[32 j + i] =
// Commit_data[i][j], main.cpp:99-103) with the separable weights v1[32 j +
// i] = brow[i] bcol[j] (the point's beta, or the input vectors' product) as
// sum_j bcol[j] sum_i brow[i] rows[p][i][j]: no 32 x len table is read.
// Per-CTA partials.
__global__ void __launch_bounds__(kRedThreads)
k_fip_partial(const fe *rows, uint64_t pstride, int nrows, uint64_t len, const fe *brow, const fe *bcol,
              fe *partial) {
  __shared__ fe red[kRedThreads];
  __shared__ fe sr[32];
  if (threadIdx.x < 32) sr[threadIdx.x] = brow[threadIdx.x];
  __syncthreads();
  fe acc = fe_zero();
  const fe *r = rows + blockIdx.y * pstride;
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < len; j += (uint64_t)gridDim.x * blockDim.x) {
    fe c = fe_zero();
    for (int i = 0; i < nrows; i++) c = fadd(c, fmul(r[(uint64_t)i * len + j], sr[i]));
    acc = fadd(acc, fmul(c, bcol[j]));
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fadd(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(uint64_t)blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// The leader's combination (MPI_utils.cpp:514-527): K = sum_p lambda_p y_p,
// thread p forming y_p (launched with at least N <= 64 threads).
__global__ void k_fip_combine(const fe *partial, int nblk, int N, const fe *lambda, fe *K) {
  __shared__ fe t[kPcsMaxParties];
  const int p = threadIdx.x;
  if (p < N) {
    fe y = fe_zero();
    for (int k = 0; k < nblk; k++) y = fadd(y, partial[(uint64_t)p * nblk + k]);
    t[p] = fmul(lambda[p], y);
  }
  __syncthreads();
  if (p) return;
  fe acc = fe_zero();
  for (int q = 0; q < N; q++) acc = fadd(acc, t[q]);
  *K = acc;
}

// A record payload copied from party-major vectors: out[p][0..len) -> tr.
__global__ void k_put_party(const fe *v, uint64_t len, int N, uint8_t *tr, uint64_t off, uint64_t rec_stride) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= len) return;
  put_fe(tr, off + blockIdx.y * rec_stride + 16 * j, v[blockIdx.y * len + j]);
}

unsigned grid(uint64_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------- coSumcheck round drivers
// quadratic_coSumcheck / cubic_coSumcheck (coSumcheck.cpp:233-448) with N
// parties on the device: per round every party's block transforms and
// products (phase 1), plus the challenge-weighted sparse vectors R, the
// leader's aggregation (sumcheck_aggr), its check and challenge, the sparse
// fold of R and the block fold of every vector (phase 2); then the final
// shares, the leader's unpack and check, the last challenge and the claims.

constexpr int kCoscMaxRounds = 16;
constexpr int kCoscMaxRows = 5;  // final values per party: 5 (quadratic) / 4 (cubic)

struct CoscDev {
  fe fs, K, c;
  uint32_t flags;   // bit i: round i's message does not match K; bit 29: final check; bit 30: b1 check
  fe r[kCoscMaxRounds];
  fe fer[kPcsMaxParties];  // final_eval_r of every party
};

// c = hash_to_field({K, K_r}), K += c K_r (coSumcheck.cpp:234-235).
__global__ void k_cosc_init(CoscDev *st, fe fs, fe K, fe Kr, uint8_t *tr, uint64_t off_c) {
  fs = hash_F(fs, K);
  fs = hash_F(fs, Kr);
  st->fs = fs;
  st->c = fs;
  st->K = fadd(K, fmul(fs, Kr));
  st->flags = 0;
  put_fe(tr, off_c, fs);
}

// Offsets of the sparse vectors R[j] of one party (R holds them back to back).
struct ROffs {
  int n;
  uint32_t off[kCoscMaxRounds + 1];
};

// H_p += c H_r with H_r = R_p[iter], H_r[0] += sum_{j > iter} sum_k R_p[j][step k]
// (coSumcheck.cpp:47-60, 181-193).  One CTA per party.
__global__ void k_cosc_add_hr(fe *H, int D, const fe *R, uint64_t rstride, ROffs ro, int iter, int step,
                              const CoscDev *st) {
  const uint64_t p = blockIdx.x;
  const fe *Rp = R + p * rstride;
  __shared__ fe extra;
  if (threadIdx.x == 0) {
    fe e = fe_zero();
    for (int j = iter + 1; j < ro.n; j++) {
      const int len = (int)(ro.off[j + 1] - ro.off[j]);
      for (int k = 0; k < len / step; k++) e = fadd(e, Rp[ro.off[j] + step * k]);
    }
    extra = e;
  }
  __syncthreads();
  const fe c = st->c;
  for (int k = threadIdx.x; k < D; k += blockDim.x) {
    fe hr = Rp[ro.off[iter] + k];
    if (k == 0) hr = fadd(hr, extra);
    H[p * D + k] = fadd(H[p * D + k], fmul(c, hr));
  }
}

// The leader's round: sum_{j<d} H[j << ext] = K (flag otherwise), r =
// hash_to_field(H), LD = compute_lagrange_coeff(r, D = d << ext), K = sum
// H LD, Ld = compute_lagrange_coeff(r, d) (coSumcheck.cpp:258-293,
// 362-396).  scratch: 2 D entries.
__global__ void __launch_bounds__(256)
k_cosc_verify(CoscDev *st, const fe *poly, int logd, int ext, int round, fe wi, fe invD, fe invd, fe *LD, fe *Ld,
              fe *scratch, uint8_t *tr, uint64_t off_poly, uint64_t off_chal) {
  __shared__ fe red[256];
  __shared__ fe chal;
  __shared__ fe sh_cw[2 * 1024];  // the powers of c and of w^-1 (global scratch beyond 1024 points)
  const int d = 1 << logd, D = d << ext;
  fe *cp = D <= 1024 ? sh_cw : scratch, *wp = D <= 1024 ? sh_cw + D : scratch + D;
  // (wi = omega_D^-1, invD, invd: constants of the shape, formed on the host)
  for (int k = threadIdx.x; k < D; k += blockDim.x) {
    wp[k] = fpow(wi, (uint64_t)k);
    put_fe(tr, off_poly + 16ull * k, poly[k]);
  }
  if (threadIdx.x == 0) {
    fe ev = fe_zero();
    for (int j = 0; j < d; j++) ev = fadd(ev, poly[j << ext]);
    if (!fe_eq(ev, st->K)) st->flags |= 1u << round;
    fe fs = st->fs;
    for (int k = 0; k < D; k++) fs = hash_F(fs, poly[k]);
    st->fs = fs;
    st->r[round] = fs;
    put_fe(tr, off_chal, fs);
    chal = fs;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < D; k += blockDim.x) cp[k] = fpow(chal, (uint64_t)k);
  __syncthreads();
  fe acc = fe_zero();
  for (int k = threadIdx.x; k < D; k += blockDim.x) {
    fe s = fe_zero();
    for (int j = 0; j < D; j++) s = fadd(s, fmul(cp[j], wp[((uint64_t)j * k) & (D - 1)]));
    s = fmul(s, invD);
    LD[k] = s;
    acc = fadd(acc, fmul(poly[k], s));
  }
  for (int k = threadIdx.x; k < d; k += blockDim.x) {
    fe s = fe_zero();
    for (int j = 0; j < d; j++) s = fadd(s, fmul(cp[j], wp[(((uint64_t)j * k) << ext) & (D - 1)]));
    Ld[k] = fmul(s, invd);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fadd(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) st->K = red[0];
}

// quadratic_coSumcheck_phase2_sparse (coSumcheck.cpp:215-228) for every party:
// s = sum_j LD[j] R_p[iter][j]; R_p[j > iter] *= LD[0]; R_p[iter+1][0] += s.
// One CTA of kCoscThreads per party.
constexpr int kCoscThreads = 256;
__global__ void __launch_bounds__(kCoscThreads)
k_cosc_sparse(fe *R, uint64_t rstride, ROffs ro, int iter, const fe *LD, int D, int N, CoscDev *st) {
  const int p = blockIdx.x;
  if (p >= N) return;
  fe *Rp = R + (uint64_t)p * rstride;
  const int len = (int)(ro.off[iter + 1] - ro.off[iter]);
  __shared__ fe red[kCoscThreads];
  fe s = fe_zero();
  for (int j = threadIdx.x; j < len && j < D; j += kCoscThreads) s = fadd(s, fmul(LD[j], Rp[ro.off[iter] + j]));
  red[threadIdx.x] = s;
  const fe l0 = LD[0];
  for (uint32_t e = ro.off[iter + 1] + threadIdx.x; e < ro.off[ro.n]; e += kCoscThreads) Rp[e] = fmul(Rp[e], l0);
  __syncthreads();
  if (threadIdx.x) return;
  s = fe_zero();
  for (int t = 0; t < kCoscThreads; t++) s = fadd(s, red[t]);
  if (iter + 1 < ro.n) Rp[ro.off[iter + 1]] = fadd(Rp[ro.off[iter + 1]], s);
  st->fer[p] = s;
}

// The coSumcheck's inner-product vector (ip_vec, coSumcheck.cpp:240-275,
// 345-381): round i's entry j is LD_i[j] times the first entry of every
// other round's LD (each round scales all other rounds' entries by its
// LD[0]).  One CTA per round.
__global__ void k_cosc_ip(const fe *LD, ROffs ro, fe *ip) {
  const int i = blockIdx.x;
  fe others = fe_one();
  for (int t = 0; t < ro.n; t++)
    if (t != i) others = fmul(others, LD[ro.off[t]]);
  for (uint32_t j = ro.off[i] + threadIdx.x; j < ro.off[i + 1]; j += blockDim.x) ip[j] = fmul(LD[j], others);
}

// The end of the round driver (coSumcheck.cpp:300-330, 399-446): the parties'
// final values, the leader's unpack (unpack_secret_share(H, N/2, N), a fixed
// N/2 x N map U), its check, the last challenge, the Lagrange weights over
// N/4 points and the claims; for the cubic form also the check of b1[0]
// against the round weights.  One CTA of kCoscThreads: the parties' values,
// the unpack and the check's terms in parallel, the Fiat-Shamir chain and
// the claims on thread 0.
__global__ void k_cosc_final(CoscDev *st, int cubic, int N, const fe *p1, const fe *p2, const fe *p3, const fe *b1,
                             uint64_t mstride, const fe *U, const fe *b2, const fe *Ld_hist, const int *logd_hist,
                             int nrounds, const fe *r1, fe *claims, uint8_t *tr, uint64_t off_shares,
                             uint64_t off_unpacked, uint64_t off_r, uint64_t off_claims) {
  const int rows = cubic ? 4 : 5, half = N / 2, quarter = N / 4;
  __shared__ fe H[kCoscMaxRows][kPcsMaxParties / 2];
  __shared__ fe S[kPcsMaxParties][kCoscMaxRows];
  __shared__ fe red[kCoscThreads];
  // the parties' final values (thread p), then the unpack (thread (i, j))
  for (int p = threadIdx.x; p < N; p += blockDim.x) {
    const uint64_t o = (uint64_t)p * mstride;
    fe *sp = S[p];
    if (cubic) {
      sp[0] = p1[o];
      sp[1] = p2[o];
      sp[2] = p3[o];
      sp[3] = st->fer[p];
    } else {
      sp[0] = p1[o];
      sp[1] = p2[o];
      sp[2] = p1[o + 1];
      sp[3] = p2[o + 1];
      sp[4] = st->fer[p];
    }
    for (int i = 0; i < rows; i++) put_fe(tr, off_shares + 16ull * ((uint64_t)p * rows + i), sp[i]);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < rows * half; q += blockDim.x) {
    const int i = q / half, j = q % half;
    fe h = fe_zero();
    for (int p = 0; p < N; p++) h = fadd(h, fmul(U[j * N + p], S[p][i]));
    H[i][j] = h;
    put_fe(tr, off_unpacked + 16ull * (i * half + j), h);
  }
  __syncthreads();
  // the cubic form's b1 check (coSumcheck.cpp:432-443): per round the d
  // terms in parallel, their sum and the product by thread 0
  fe y = fe_one();
  if (cubic) {
    int ctr = 0, at = 0;
    for (int i = 0; i < nrounds; i++) {
      const int ld = logd_hist[i], d = 1 << ld;
      fe acc = fe_zero();
      for (int j = threadIdx.x; j < d; j += blockDim.x) {
        fe b = fe_one();
        for (int t = 0; t < ld; t++) b = fmul(b, ((j >> t) & 1) ? r1[ctr + t] : fsub(fe_one(), r1[ctr + t]));
        acc = fadd(acc, fmul(b, Ld_hist[at + j]));
      }
      red[threadIdx.x] = acc;
      __syncthreads();
      if (threadIdx.x == 0) {
        fe a = fe_zero();
        for (int t = 0; t < (int)blockDim.x; t++) a = fadd(a, red[t]);
        y = fmul(y, a);
      }
      __syncthreads();
      ctr += ld;
      at += d;
    }
  }
  if (threadIdx.x) return;
  fe K = st->K;
  const fe c = st->c;
  for (int i = 0; i < quarter; i++) {
    fe t;
    if (cubic) t = fmul(b2[i], fadd(fmul(b1[0], fsub(fmul(H[0][i], H[1][i]), H[2][i])), fmul(c, H[3][i])));
    else t = fadd(fadd(fmul(H[0][i], H[1][i]), fmul(H[2][i], H[3][i])), fmul(c, H[4][i]));
    K = fsub(K, t);
  }
  if (!fe_eq(K, fe_zero())) st->flags |= 1u << 29;
  fe fs = st->fs;
  const int hashed = cubic ? 3 : rows;
  for (int i = 0; i < hashed; i++)
    for (int j = 0; j < half; j++) fs = hash_F(fs, H[i][j]);
  st->fs = fs;
  put_fe(tr, off_r, fs);
  // L over N/4 points: compute_lagrange_coeff(r, N/4), or {1} for one point
  fe L[kPcsMaxParties / 4];
  if (quarter == 1) {
    L[0] = fe_one();
  } else {
    int lq = 0;
    while ((1 << lq) < quarter) lq++;
    const fe wi = finv(root_of_unity(lq)), iq = finv(fe_make((uint64_t)quarter, 0));
    for (int k = 0; k < quarter; k++) {
      fe acc = fe_zero(), x = fe_one();
      const fe step = fpow(wi, (uint64_t)k);
      fe w = fe_one();
      for (int j = 0; j < quarter; j++) {
        acc = fadd(acc, fmul(x, w));
        x = fmul(x, fs);
        w = fmul(w, step);
      }
      L[k] = fmul(acc, iq);
    }
  }
  for (int i = 0; i < rows; i++) {
    fe e = fe_zero();
    for (int j = 0; j < quarter; j++) e = fadd(e, fmul(L[j], H[i][j]));
    claims[i] = e;
    put_fe(tr, off_claims + 16ull * i, e);
  }
  if (cubic && !fe_eq(y, b1[0])) st->flags |= 1u << 30;
}

}  // namespace
}  // namespace gbz

// ------------------------------------------------------------ host side

using namespace gbz;

namespace {

// prepare_parameters (coPCS.cpp:38-72) with get_degrees / get_queries
// (New_PCS.cpp:23-77).  The query counts are the reference's double
// expressions, truncated as it truncates them.
struct PcsSchedule {
  int N = 0, rounds = 0;
  uint64_t M = 0;
  std::vector<int> rate0, rate1, degrees, queries, delegation;
  int log_rate_offset = 0;
  uint64_t randomness = 0;  // sum_i queries[i] degrees[i]
};

PcsSchedule make_schedule(int N, uint64_t M, int rounds, const int *rate0, const int *rate1) {
  if (N < 4 || N > kPcsMaxParties || !is_pow2((uint64_t)N)) throw ArgError("pcs: N must be a power of two in [4, 64]");
  if (rounds < 3 || rounds > kPcsMaxRounds) throw ArgError("pcs: 3..8 rounds (rates)");
  if (!is_pow2(M)) throw ArgError("pcs: M must be a power of two");
  PcsSchedule s;
  s.N = N;
  s.M = M;
  s.rounds = rounds;
  for (int i = 0; i < rounds; i++) {
    if (rate0[i] < 2 || !is_pow2((uint64_t)rate0[i])) throw ArgError("pcs: tensor rates must be powers of two >= 2");
    s.rate0.push_back(rate0[i]);
    const int r1 = i >= 2 ? rate1[i] : 0;
    if (i >= 2 && (r1 < 2 || !is_pow2((uint64_t)r1))) throw ArgError("pcs: row rates must be powers of two >= 2");
    s.rate1.push_back(r1);
  }
  const uint64_t row_size = 2 * (4 * M / (uint64_t)N);
  int log_size = ilog2(row_size);
  s.degrees.push_back(32);
  log_size -= 5;
  s.degrees.push_back(8);
  log_size -= 3;
  const int deg = log_size / (rounds - 2);
  if (log_size < 1 || deg < 1) throw ArgError("pcs: M too small for the degree schedule");
  for (int i = 1; i < rounds - 2; i++) s.degrees.push_back(1 << deg);
  s.degrees.push_back(1 << (log_size - deg * (rounds - 3)));
  for (int i = 0; i < rounds; i++) {
    volatile double q;
    if (i <= 1) {
      volatile double t = 1.0 - 1.0 / (double)rate0[0];
      volatile double u = 0.25 * t;
      volatile double v = 1 - u;
      q = 100.0 / (-std::log2(v));
      s.queries.push_back((int)q);
    } else {
      volatile double a = 1.0 - 1.0 / (double)rate0[i];
      volatile double sq = std::sqrt(1.0 / (double)s.rate1[i]);
      volatile double b = 0.5 * 0.5 * a;
      volatile double c = b * (1 - sq);
      volatile double e1 = 1 - c;
      const int l1 = (int)(100.0 / (-std::log2(e1)));
      volatile double e2 = 1 - b;
      volatile double t1 = 100.0 / (-std::log2(e2));
      volatile double t2 = 100.0 / (-std::log2(sq));
      volatile double t3 = t1 + t2;
      const int l2 = (int)t3;
      s.queries.push_back(l1 > l2 ? l2 : l1);
    }
  }
  int ro = 1;
  for (int i = 1; i < rounds; i++) ro *= rate0[i];
  s.log_rate_offset = ilog2((uint64_t)ro);
  for (int i = 2; i < rounds; i++) {
    uint64_t x = (uint64_t)s.degrees[i] * s.queries[i], p2 = 1;
    while (p2 < x) p2 <<= 1;
    s.delegation.push_back((int)p2);
  }
  for (int i = 0; i < rounds; i++) s.randomness += (uint64_t)s.queries[i] * s.degrees[i];
  for (int i = 0; i < rounds; i++)
    if (s.queries[i] < 1 || s.queries[i] > kPcsMaxQueries) throw ArgError("pcs: 1..1024 queries per round");
  for (int i = 1; i < rounds; i++)
    if (s.degrees[i] > (1 << kPcsMaxLogDeg)) throw ArgError("pcs: round degree above 2^10");
  return s;
}

// One copy run of prepare_data (coPCS.cpp:76-129): `count` entries of the
// shares (src 0) or the random shares (src 1) from src_off into row `row`
// at column `col`.
struct Run {
  int row;
  uint64_t col;
  int src;
  uint64_t src_off, count;
};

std::vector<Run> prepare_runs(uint64_t S, uint64_t R, uint64_t Bs, uint64_t q0, int *batches) {
  if (q0 >= Bs) throw ArgError("pcs: the first round's queries fill a whole row (M too small)");
  std::vector<Run> runs;
  uint64_t dc = 0, rc = 0;
  int last = -1;
  for (int i = 0; i < 32; i++) {
    const uint64_t take = std::min(Bs - q0, S - dc);
    runs.push_back({i, 0, 0, dc, take});
    dc += take;
    if (rc + q0 > R) throw ArgError("pcs: too few random shares");
    runs.push_back({i, Bs - q0, 1, rc, q0});
    rc += q0;
    if (dc == S) {
      last = i;
      break;
    }
  }
  if (dc < S || last + 1 >= 32) throw ArgError("pcs: more batches are needed (M too large for 32 rows)");
  const int lr = last + 1;
  uint64_t count;
  // The reference compares Shares.size() - rand_ctr as an unsigned value, so
  // rand_ctr > Shares.size() takes the first case too.
  if (S < rc || S - rc > Bs) {
    if (rc >= R) throw ArgError("pcs: too few random shares");
    count = std::min(Bs, R - rc);
  } else {
    count = Bs - (S - rc);
    if (count > R - rc) throw ArgError("pcs: too few random shares");
  }
  runs.push_back({lr, 0, 1, rc, count});
  *batches = lr + 1;
  return runs;
}

// Packed-Shamir constants of N parties: the share map (compute_secret_shares)
// and the tensor scales of tensor_eval_vector; both depend on N only.
fe host_tensor_scale(uint32_t p0, int cols, int my_id) {
  const int lg4 = ilog2(4ull * (uint64_t)cols);
  const fe w2 = fpow(root_of_unity(lg4), 2ull * p0 + 1);
  const fe step = fpow(root_of_unity(lg4), 2ull * (uint64_t)my_id + 1);
  std::vector<fe> pw(cols);
  fe x = fe_one();
  for (int t = 0; t < cols; t++) {
    pw[t] = x;
    x = fmul(x, w2);
  }
  fe acc = fe_zero(), e = fe_one();
  for (int t = 0; t < cols; t++) {
    acc = fadd(acc, fmul(pw[(cols - t) % cols], e));
    e = fmul(e, step);
  }
  return fmul(acc, finv(fe_make((uint64_t)cols, 0)));
}

}  // namespace

struct gbz_pcs {
  int device = 0;
  PcsSchedule sc;
  uint64_t S = 0, R = 0, Bs = 0, L = 0;  // share length, random length, row length, codeword length
  int batches = 0;
  fe *cd = nullptr;      // [N][batches][Bs] Commit_data
  fe *cw = nullptr;      // [N][batches][L] codewords
  uint8_t *levels = nullptr;  // [N][2L - 1] column-root trees of distributed_MT
  uint8_t *roots = nullptr;   // [N][32] party roots, then [N][32] the leader root each party derives
  std::vector<void *> owned;

  ~gbz_pcs() {
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    for (void *p : owned) cudaFree(p);
    if (prev >= 0) cudaSetDevice(prev);
  }
  template <typename T>
  T *alloc(uint64_t count) {
    void *p = nullptr;
    GBZ_CUDA(cudaMalloc(&p, std::max<uint64_t>(count * sizeof(T), 16)));
    owned.push_back(p);
    return (T *)p;
  }
};

namespace {

// The record layout of an opening: header list and the payload offsets.
struct PcsLayout {
  std::vector<Hdr> hdr;
  uint64_t bytes = 0;
  uint64_t add(uint32_t tag, uint32_t count, uint64_t unit) {
    hdr.push_back({bytes, tag, count});
    const uint64_t payload = bytes + 8;
    bytes += 8 + unit * count;
    return payload;
  }
};

struct RoundOffs {
  uint64_t pp, poly, chal, roots, leader, queries, y, seg, s, K;
};
struct OpenOffs {
  uint64_t pp0, poly0, chal0, K0, broots, bleader, bqueries, final_;
  std::vector<RoundOffs> r;
};

OpenOffs open_layout(const gbz_pcs &pc, PcsLayout &lay) {
  const PcsSchedule &sc = pc.sc;
  const int N = sc.N;
  OpenOffs o;
  o.pp0 = lay.add(T_PCS_PARTY_POLYS, 3 * N, 16);
  o.poly0 = lay.add(T_PCS_POLY, 3, 16);
  o.chal0 = lay.add(T_PCS_CHALLENGE, 1, 16);
  o.K0 = lay.add(T_PCS_K, 1, 16);
  o.broots = lay.add(T_PCS_ROOTS, N, 32);
  o.bleader = lay.add(T_PCS_LEADER_ROOT, 1, 32);
  o.bqueries = lay.add(T_PCS_QUERIES, 2 * sc.queries[0], 4);
  for (int i = 0; i + 1 < sc.rounds; i++) {
    const int d = sc.degrees[i + 1], l = sc.queries[i + 1];
    RoundOffs r;
    r.pp = lay.add(T_PCS_PARTY_POLYS, 2 * d * N, 16);
    r.poly = lay.add(T_PCS_POLY, 2 * d, 16);
    r.chal = lay.add(T_PCS_CHALLENGE, 1, 16);
    r.roots = lay.add(T_PCS_ROOTS, N, 32);
    r.leader = lay.add(T_PCS_LEADER_ROOT, 1, 32);
    r.queries = lay.add(T_PCS_QUERIES, 2 * l, 4);
    r.y = lay.add(T_PCS_Y, l, 16);
    r.seg = lay.add(T_PCS_SEGMENTS, l * d, 16);
    r.s = lay.add(T_PCS_S, 1, 16);
    r.K = lay.add(T_PCS_K, 1, 16);
    o.r.push_back(r);
  }
  // final: per party bcd, B, C' (send_pcs_data, MPI_utils.cpp:58-116)
  uint64_t n = pc.Bs, cpl = pc.L;
  for (int i = 0; i + 1 < sc.rounds; i++) {
    const uint64_t d = sc.degrees[i + 1];
    n /= d;
    cpl = (i + 2 < sc.rounds) ? n * sc.rate0[i + 2] : cpl / d;
  }
  o.final_ = lay.add(T_PCS_FINAL, (uint32_t)(N * (2 * n + cpl)), 16);
  return o;
}

// The sizes of the leader's tail (pointers are filled in by the opening).
// The PIOP mode's inputs (gbz_pcs_open_piop; the caller's memory kind).
struct PiopIn {
  const uint64_t *b1 = nullptr, *b2 = nullptr, *b3 = nullptr, *lag = nullptr;
  int nb1 = 0, nb3 = 0, nlag = 0;
  uint64_t nb2 = 0;
  const int *loglag = nullptr;
  gbz_whir_slot *slots = nullptr;
};

LeaderInputs leader_shape(const gbz_pcs &pc, const PiopIn *pi = nullptr) {
  const PcsSchedule &sc = pc.sc;
  LeaderInputs in;
  if (pi) {
    if (pi->nlag < 1 || pi->nlag > 8) throw ArgError("pcs: 1..8 Lagrange factors");
    in.piop = true;
    in.nlag = pi->nlag;
    for (int k = 0; k < pi->nlag; k++) in.loglag[k] = pi->loglag[k];
    in.q0 = (uint64_t)sc.queries[0];
  }
  in.N = sc.N;
  in.Bs = pc.Bs;
  in.log_rate_offset = sc.log_rate_offset;
  in.rate0 = sc.rate0;
  uint64_t n = pc.Bs, cpl = pc.L;
  for (int i = 0; i + 1 < sc.rounds; i++) {
    LeaderRound r;
    r.d = sc.degrees[i + 1];
    r.l = sc.queries[i + 1];
    r.n = cpl;
    r.C0 = i ? (uint64_t)sc.degrees[i + 1] * sc.rate1[i + 1] : 0;
    r.rate_next = i + 2 < sc.rounds ? sc.rate0[i + 2] : 0;
    r.rate_cur = sc.rate0[i + 1];
    in.rounds.push_back(r);
    n /= (uint64_t)r.d;
    cpl = (i + 2 < sc.rounds) ? n * sc.rate0[i + 2] : cpl / r.d;
  }
  in.n_final = n;
  in.cpl_final = cpl;
  in.max_delegation = 0;
  for (int v : sc.delegation) in.max_delegation = std::max<uint64_t>(in.max_delegation, (uint64_t)v);
  return in;
}

// The records of the leader's tail after the parties' records (lay.bytes is
// where they start), and its draws (script, arena_len: may be null).
void tail_layout(const gbz_pcs &pc, PcsLayout &lay, std::vector<DrawOp> *script = nullptr,
                 uint64_t *arena_len = nullptr, const PiopIn *pi = nullptr) {
  LeaderInputs in = leader_shape(pc, pi);
  Layout tl;
  tl.record_headers = true;
  LeaderResources R;
  leader_tail(R, in, nullptr, nullptr, nullptr, tl, script, arena_len, nullptr);
  const uint64_t base = lay.bytes;
  for (const auto &h : tl.headers) lay.hdr.push_back({base + h.off, h.tag, h.count});
  lay.bytes = base + tl.len;
}

}  // namespace

namespace gbz {

CoscOut cosumcheck_run(gbz_ctx *ctx, int form, int N, uint64_t n, const fe *p1, const fe *p2, const fe *p3,
                       const fe *R, cudaMemcpyKind kin, const fe *r1, int nr1, const fe *r2, fe hK, fe hKr,
                       const int *degrees, int ndeg, fe hfs, uint8_t *transcript, cudaMemcpyKind tr_kind, fe *ip) {
  if (form != GBZ_SC_QUADRATIC && form != GBZ_SC_CUBIC) throw ArgError("coSumcheck: form must be quadratic or cubic");
  const bool cubic = form == GBZ_SC_CUBIC;
  if (cubic && (!p3 || !r1)) throw ArgError("coSumcheck: the cubic form needs p3 and r1");
  if (N < 4 || N > kPcsMaxParties || !is_pow2((uint64_t)N)) throw ArgError("coSumcheck: N must be a power of two in [4, 64]");
  if (ndeg < 1 || ndeg > kCoscMaxRounds) throw ArgError("coSumcheck: 1..16 rounds");
  check_pow2(n, "coSumcheck: n");
  const int ext = cubic ? 2 : 1, step = 1 << ext, rows = cubic ? 4 : 5;
  uint64_t m = n;
  std::vector<int> logd(ndeg);
  ROffs ro{};
  ro.n = ndeg;
  ro.off[0] = 0;
  for (int i = 0; i < ndeg; i++) {
    if (degrees[i] < 1 || !is_pow2((uint64_t)degrees[i]) || degrees[i] > 1024 || (uint64_t)degrees[i] > m)
      throw ArgError("coSumcheck: degrees must be powers of two <= 1024 dividing the length");
    logd[i] = ilog2((uint64_t)degrees[i]);
    m /= degrees[i];
    ro.off[i + 1] = ro.off[i] + (uint32_t)(step * degrees[i]);
  }
  if (m < (cubic ? 1u : 2u)) throw ArgError("coSumcheck: the folds must leave 2 (quadratic) / 1 (cubic) entries");
  const int lq = ilog2((uint64_t)(N / 4));
  if (cubic && (nr1 < 0 || (1ull << nr1) != n)) throw ArgError("coSumcheck: r1 must have log2(n) entries");
  // transcript layout
  PcsLayout lay;
  const uint64_t off_c = lay.add(T_PCS_CHALLENGE, 1, 16);
  std::vector<uint64_t> off_pp(ndeg), off_poly(ndeg), off_chal(ndeg);
  for (int i = 0; i < ndeg; i++) {
    const int D = degrees[i] << ext;
    off_pp[i] = lay.add(T_PCS_PARTY_POLYS, D * N, 16);
    off_poly[i] = lay.add(T_PCS_POLY, D, 16);
    off_chal[i] = lay.add(T_PCS_CHALLENGE, 1, 16);
  }
  const uint64_t off_sh = lay.add(T_COSC_FINAL_SHARES, rows * N, 16);
  const uint64_t off_un = lay.add(T_COSC_UNPACKED, rows * (N / 2), 16);
  const uint64_t off_r = lay.add(T_PCS_CHALLENGE, 1, 16);
  const uint64_t off_cl = lay.add(T_COSC_CLAIMS, rows, 16);
  cudaStream_t s = ctx->stream;
  OpenBufs ob;
  {
    std::string key = "cosumcheck:" + std::to_string(form) + ":" + std::to_string(N) + ":" + std::to_string(n) + ":" +
                      std::to_string((int)kin) + ":" + std::to_string(transcript != nullptr) + ":" + std::to_string(ip != nullptr);
    for (int i = 0; i < ndeg; i++) key += ":" + std::to_string(degrees[i]);
    ob.pool = &ctx->pools[key];
  }
  // party-major inputs, copied: the call folds them in place as the reference does
  const uint64_t Rst = ro.off[ndeg];
  fe *v1 = ob.alloc<fe>((uint64_t)N * n), *v2 = ob.alloc<fe>((uint64_t)N * n), *v3 = nullptr, *vb = nullptr;
  fe *dR = ob.alloc<fe>((uint64_t)N * Rst);
  GBZ_CUDA(cudaMemcpyAsync(v1, p1, 16ull * N * n, kin, s));
  GBZ_CUDA(cudaMemcpyAsync(v2, p2, 16ull * N * n, kin, s));
  GBZ_CUDA(cudaMemcpyAsync(dR, R, 16ull * N * Rst, kin, s));
  // the quadratic form takes no points (r1, r2 may be null there)
  std::vector<fe> hr1(cubic ? r1 : nullptr, cubic ? r1 + nr1 : nullptr), hr2(lq, fe_zero());
  if (cubic && lq) hr2.assign(r2, r2 + lq);
  if (cubic) {
    v3 = ob.alloc<fe>((uint64_t)N * n);
    vb = ob.alloc<fe>((uint64_t)N * n);
    GBZ_CUDA(cudaMemcpyAsync(v3, p3, 16ull * N * n, kin, s));
  }
  // b1 = precompute_beta(r1) for every party (the same vector), b2 = precompute_beta(r2)
  std::vector<fe> b2(N / 4, fe_one());
  for (int i = 0; i < N / 4; i++) {
    fe v = fe_one();
    for (int t = 0; t < lq; t++) v = fmul(v, ((i >> t) & 1) ? hr2[t] : fsub(fe_one(), hr2[t]));
    b2[i] = v;
  }
  fe *dr1 = ob.alloc<fe>(std::max(1, nr1)), *db2 = ob.alloc<fe>(N / 4);
  GBZ_CUDA(cudaMemcpyAsync(db2, b2.data(), 16ull * (N / 4), cudaMemcpyHostToDevice, s));
  if (cubic) {
    GBZ_CUDA(cudaMemcpyAsync(dr1, hr1.data(), 16ull * nr1, cudaMemcpyHostToDevice, s));
    beta_launch(dr1, nr1, vb, s);
    for (int p = 1; p < N; p++) GBZ_CUDA(cudaMemcpyAsync(vb + (uint64_t)p * n, vb, 16 * n, cudaMemcpyDeviceToDevice, s));
  }
  // sumcheck_aggr's weights: ones (quadratic, coSumcheck.cpp:194) or b2 (cubic)
  std::vector<fe> ones(N / 4, fe_one());
  std::vector<fe> lambda = aggregate_weights(N, cubic ? b2.data() : ones.data());
  // unpack_secret_share(H, N/2, N): row j of the map takes E[2j]
  std::vector<fe> U((size_t)(N / 2) * N);
  for (int j = 0; j < N / 2; j++) {
    std::vector<fe> g(N, fe_zero());
    g[2 * j] = fe_one();
    std::vector<fe> l = aggregate_weights_even(N, g);
    for (int p = 0; p < N; p++) U[(size_t)j * N + p] = l[p];
  }
  fe *dl = ob.alloc<fe>(N), *dU = ob.alloc<fe>(U.size());
  GBZ_CUDA(cudaMemcpyAsync(dl, lambda.data(), 16ull * N, cudaMemcpyHostToDevice, s));
  GBZ_CUDA(cudaMemcpyAsync(dU, U.data(), 16 * U.size(), cudaMemcpyHostToDevice, s));
  uint8_t *tr = ob.alloc<uint8_t>(lay.bytes);
  Hdr *dh = ob.alloc<Hdr>(lay.hdr.size());
  GBZ_CUDA(cudaMemcpyAsync(dh, lay.hdr.data(), sizeof(Hdr) * lay.hdr.size(), cudaMemcpyHostToDevice, s));
  k_headers<<<grid(lay.hdr.size()), 256, 0, s>>>(dh, (int)lay.hdr.size(), tr);
  CoscDev *st = ob.alloc<CoscDev>(1);
  k_cosc_init<<<1, 1, 0, s>>>(st, hfs, hK, hKr, tr, off_c);
  GBZ_CUDA(cudaGetLastError());
  const int maxD = 1024 << ext;
  // every round's Lagrange vector over its extended block, kept for ip_vec
  fe *H = ob.alloc<fe>((uint64_t)N * maxD), *poly = ob.alloc<fe>(maxD), *LDall = ob.alloc<fe>(ro.off[ndeg]);
  fe *scr = ob.alloc<fe>(2ull * maxD), *coef = ob.alloc<fe>((uint64_t)N * n);
  uint64_t dsum = 0;
  for (int i = 0; i < ndeg; i++) dsum += degrees[i];
  fe *Ldh = ob.alloc<fe>(dsum);
  int *dlog = ob.alloc<int>(ndeg);
  GBZ_CUDA(cudaMemcpyAsync(dlog, logd.data(), 4ull * ndeg, cudaMemcpyHostToDevice, s));
  m = n;
  uint64_t at = 0;
  for (int i = 0; i < ndeg; i++) {
    const int d = degrees[i], D = d << ext;
    const uint64_t blocks = (uint64_t)N * m / d, pblocks = m / d;
    // phase 1 (coSumcheck.cpp:9-46, 150-179): extended blocks of every vector
    const NttTables &td = ctx->tables(logd[i]), &tD = ctx->tables(logd[i] + ext);
    if (logd[i] + ext > kMaxCoLogD) throw ArgError("coSumcheck: extended block longer than 2^13");
    fe *src[4] = {v1, v2, cubic ? vb : nullptr, cubic ? v3 : nullptr};
    fe *ex[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int v = 0; v < (cubic ? 4 : 2); v++) {
      ex[v] = ob.alloc<fe>(blocks * D);
      ntt_batched(td, src[v], d, (uint32_t)d, coef, blocks, true, s);
      ntt_batched(tD, coef, d, (uint32_t)d, ex[v], blocks, false, s);
    }
    uint8_t *zf = nullptr;
    if (cubic) {  // blocks whose p1 part is all zero are skipped (coSumcheck.cpp:21-27)
      zf = ob.alloc<uint8_t>(blocks);
      nonzero_blocks_launch(v1, blocks, logd[i], zf, s);
    }
    const int lanes = D >= 256 ? 1 : 256 / D;
    const int per_cta = (int)std::max<uint64_t>((uint64_t)lanes, (pblocks + 607) / 608);
    fe *cpart = ob.alloc<fe>((uint64_t)N * D * cophase1_parts(pblocks, per_cta));
    cophase1_reduce_launch(ex[0], ex[1], ex[2], ex[3], zf, pblocks, logd[i] + ext, per_cta, cpart, H, s, N);
    k_cosc_add_hr<<<N, 256, 0, s>>>(H, D, dR, Rst, ro, i, step, st);
    k_put_party<<<dim3(grid(D), N), 256, 0, s>>>(H, D, N, tr, off_pp[i], 16ull * D);
    aggregate_launch(H, N, D, dl, poly, s);
    fe *LD = LDall + ro.off[i];
    k_cosc_verify<<<1, 256, 0, s>>>(st, poly, logd[i], ext, i, finv(root_of_unity(logd[i] + ext)),
                                    finv(fe_make((uint64_t)D, 0)), finv(fe_make(1ull << logd[i], 0)), LD, Ldh + at,
                                    scr, tr, off_poly[i], off_chal[i]);
    k_cosc_sparse<<<N, kCoscThreads, 0, s>>>(dR, Rst, ro, i, LD, D, N, st);
    GBZ_CUDA(cudaGetLastError());
    // phase 2 (coSumcheck.cpp:66-148, 201-213): every vector folded by Ld
    for (fe *v : {v1, v2, v3, vb}) {
      if (!v) continue;
      cophase2_launch(v, (uint64_t)N * m, Ldh + at, logd[i], coef, s);
      GBZ_CUDA(cudaMemcpyAsync(v, coef, 16ull * N * m / d, cudaMemcpyDeviceToDevice, s));
    }
    m /= d;
    at += d;
  }
  fe *dcl = ob.alloc<fe>(rows);
  k_cosc_final<<<1, kCoscThreads, 0, s>>>(st, cubic ? 1 : 0, N, v1, v2, v3, vb, m, dU, db2, Ldh, dlog, ndeg, dr1, dcl, tr,
                                off_sh, off_un, off_r, off_cl);
  GBZ_CUDA(cudaGetLastError());
  if (ip) {
    k_cosc_ip<<<ndeg, 256, 0, s>>>(LDall, ro, ip);
    GBZ_CUDA(cudaGetLastError());
  }
  CoscDev hst;
  GBZ_CUDA(cudaMemcpyAsync(&hst, st, sizeof(CoscDev), cudaMemcpyDeviceToHost, s));
  std::vector<fe> hcl(rows);
  GBZ_CUDA(cudaMemcpyAsync(hcl.data(), dcl, 16ull * rows, cudaMemcpyDeviceToHost, s));
  if (transcript) GBZ_CUDA(cudaMemcpyAsync(transcript, tr, lay.bytes, tr_kind, s));
  GBZ_CUDA(cudaStreamSynchronize(s));
  // claims: rows x (eval, r vector [r_final, r_0, ..., r_{ndeg-1}])
  CoscOut out;
  out.claims.resize((size_t)rows * (ndeg + 2));
  for (int i = 0; i < rows; i++) {
    fe *o = out.claims.data() + (size_t)i * (ndeg + 2);
    o[0] = hcl[i];
    o[1] = hst.fs;
    for (int k = 0; k < ndeg; k++) o[2 + k] = hst.r[k];
  }
  out.fs = hst.fs;
  out.flags = hst.flags;
  return out;
}

uint64_t cosumcheck_bytes(int form, int N, const int *degrees, int ndeg) {
  if (!degrees || ndeg < 1 || N < 4) return 0;
  const int ext = form == GBZ_SC_CUBIC ? 2 : 1, rows = form == GBZ_SC_CUBIC ? 4 : 5;
  PcsLayout lay;
  lay.add(T_PCS_CHALLENGE, 1, 16);
  for (int i = 0; i < ndeg; i++) {
    lay.add(T_PCS_PARTY_POLYS, (degrees[i] << ext) * N, 16);
    lay.add(T_PCS_POLY, degrees[i] << ext, 16);
    lay.add(T_PCS_CHALLENGE, 1, 16);
  }
  lay.add(T_COSC_FINAL_SHARES, rows * N, 16);
  lay.add(T_COSC_UNPACKED, rows * (N / 2), 16);
  lay.add(T_PCS_CHALLENGE, 1, 16);
  lay.add(T_COSC_CLAIMS, rows, 16);
  return lay.bytes;
}

}  // namespace gbz

extern "C" {

gbz_status gbz_pcs_schedule(int N, uint64_t M, int rounds, const int *rate0, const int *rate1, int *degrees,
                            int *queries, uint64_t *random_per_party) {
  try {
    if (!rate0 || !rate1) return GBZ_EINVAL;
    PcsSchedule s = make_schedule(N, M, rounds, rate0, rate1);
    for (int i = 0; i < rounds; i++) {
      if (degrees) degrees[i] = s.degrees[i];
      if (queries) queries[i] = s.queries[i];
    }
    if (random_per_party) *random_per_party = s.randomness;
  } catch (const ArgError &) {
    return GBZ_EINVAL;
  }
  return GBZ_OK;
}

gbz_status gbz_pcs_commit(gbz_ctx *ctx, int N, uint64_t M, int rounds, const int *rate0, const int *rate1,
                          const uint64_t *shares, const uint64_t *random, int mem, gbz_pcs **out,
                          uint8_t *party_roots, uint8_t *leader_root) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(rate0, "rate0");
  need(rate1, "rate1");
  need(shares, "shares");
  need(random, "random");
  need(out, "out");
  *out = nullptr;
  std::unique_ptr<gbz_pcs> pc(new gbz_pcs());
  pc->device = ctx->device;
  pc->sc = make_schedule(N, M, rounds, rate0, rate1);
  const PcsSchedule &sc = pc->sc;
  pc->S = 4 * M / (uint64_t)N;
  pc->R = sc.randomness;
  pc->Bs = pc->S / 16;
  if (pc->Bs < 4) throw ArgError("pcs: shares shorter than 64 entries");
  pc->L = pc->Bs * (uint64_t)sc.rate0[0];
  if (ilog2(pc->L) > kMaxNttLogN || 1 + sc.log_rate_offset + ilog2(pc->Bs) > kMaxLogN)
    throw ArgError("pcs: codeword above 2^26");
  std::vector<Run> runs = prepare_runs(pc->S, pc->R, pc->Bs, sc.queries[0], &pc->batches);
  const uint64_t Bs = pc->Bs, L = pc->L, S = pc->S, R = pc->R;
  const int nb = pc->batches;
  cudaStream_t s = ctx->stream;
  // inputs on the device
  const fe *dsh = dev_view(ctx, 0, (const fe *)shares, 16 * S * N, mem, true);
  const fe *drn = dev_view(ctx, 1, (const fe *)random, 16 * R * N, mem, true);
  pc->cd = pc->alloc<fe>((uint64_t)N * nb * Bs);
  pc->cw = pc->alloc<fe>((uint64_t)N * nb * L);
  pc->levels = pc->alloc<uint8_t>(32ull * N * (2 * L - 1));
  pc->roots = pc->alloc<uint8_t>(64ull * N);
  // prepare_data: the rows of every party as 2-D copies (height = parties)
  GBZ_CUDA(cudaMemsetAsync(pc->cd, 0, 16ull * N * nb * Bs, s));
  for (const Run &r : runs) {
    if (!r.count) continue;
    const fe *src = (r.src ? drn : dsh) + r.src_off;
    fe *dst = pc->cd + (uint64_t)r.row * Bs + r.col;
    GBZ_CUDA(cudaMemcpy2DAsync(dst, 16 * nb * Bs, src, 16 * (r.src ? R : S), 16 * r.count, N,
                               cudaMemcpyDeviceToDevice, s));
  }
  // Encode (coPCS.cpp:131-147): every party's rows in the same launches
  encode_rows_device(ctx, pc->cd, N * nb, ilog2(Bs), sc.rate0[0], sc.log_rate_offset, pc->cw);
  // distributed_MT (coPCS.cpp:152-202) per party
  column_merkle_launch(pc->cw, nb, L, pc->levels, ilog2(N), pc->roots + 32ull * N, s, N, (uint64_t)nb * L);
  GBZ_CUDA(cudaMemcpy2DAsync(pc->roots, 32, pc->levels + 32 * (2 * L - 2), 32 * (2 * L - 1), 32, N,
                             cudaMemcpyDeviceToDevice, s));
  if (party_roots) {
    if (mem == GBZ_MEM_HOST) GBZ_CUDA(cudaMemcpyAsync(party_roots, pc->roots, 32ull * N, cudaMemcpyDeviceToHost, s));
    else GBZ_CUDA(cudaMemcpyAsync(party_roots, pc->roots, 32ull * N, cudaMemcpyDeviceToDevice, s));
  }
  if (leader_root) {
    const cudaMemcpyKind k = mem == GBZ_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    GBZ_CUDA(cudaMemcpyAsync(leader_root, pc->roots + 32ull * N, 32, k, s));
  }
  GBZ_CUDA(cudaStreamSynchronize(s));  // the staged inputs are scratch of the context
  *out = pc.release();
  API_END(ctx)
}

void gbz_pcs_free(gbz_pcs *pcs) { delete pcs; }

gbz_status gbz_pcs_info(const gbz_pcs *pcs, int *batches, uint64_t *row_len, uint64_t *codeword_len,
                        uint64_t *open_transcript_bytes) {
  if (!pcs) return GBZ_EINVAL;
  if (batches) *batches = pcs->batches;
  if (row_len) *row_len = pcs->Bs;
  if (codeword_len) *codeword_len = pcs->L;
  if (open_transcript_bytes) {
    PcsLayout lay;
    open_layout(*pcs, lay);
    *open_transcript_bytes = lay.bytes;
  }
  return GBZ_OK;
}

gbz_status gbz_pcs_commit_data(gbz_ctx *ctx, const gbz_pcs *pcs, int party, uint64_t *rows, uint64_t *codewords,
                               uint8_t *levels, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(pcs, "pcs");
  if (party < 0 || party >= pcs->sc.N) throw ArgError("pcs: party out of range");
  const cudaMemcpyKind k = mem == GBZ_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  const uint64_t nb = pcs->batches, Bs = pcs->Bs, L = pcs->L;
  if (rows) GBZ_CUDA(cudaMemcpyAsync(rows, pcs->cd + party * nb * Bs, 16 * nb * Bs, k, ctx->stream));
  if (codewords) GBZ_CUDA(cudaMemcpyAsync(codewords, pcs->cw + party * nb * L, 16 * nb * L, k, ctx->stream));
  if (levels)
    GBZ_CUDA(cudaMemcpyAsync(levels, pcs->levels + 32ull * party * (2 * L - 1), 32 * (2 * L - 1), k, ctx->stream));
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_pcs_claim(gbz_ctx *ctx, const gbz_pcs *pcs, const uint64_t *r, int nr, uint64_t *K, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(pcs, "pcs");
  need(r, "r");
  need(K, "K");
  if (pcs->device != ctx->device) throw ArgError("pcs: committed on another device");
  const int N = pcs->sc.N, nb = pcs->batches, lk = ilog2(N / 4), logBs = ilog2(pcs->Bs);
  if (nr != lk + 5 + logBs) throw ArgError("pcs: the point must have log2(N/4) + 5 + log2(row length) entries");
  cudaStream_t s = ctx->stream;
  std::vector<fe> hr(nr);
  if (mem == GBZ_MEM_DEVICE) {
    GBZ_CUDA(cudaMemcpyAsync(hr.data(), r, 16ull * nr, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaStreamSynchronize(s));
  } else {
    for (int i = 0; i < nr; i++) hr[i] = fe_make(r[2 * i], r[2 * i + 1]);
  }
  // b2 = precompute_beta(r[0 .. log2(N/4))) weights the unpacked shares
  // (MPI_utils.cpp:525-527): the same form as sumcheck_aggr's, g[2i] = b2[i]
  std::vector<fe> b2(N / 4, fe_one());
  for (int i = 0; i < (1 << lk); i++) {
    fe v = fe_one();
    for (int t = 0; t < lk; t++) {
      const fe x = hr[t];
      v = fmul(v, ((i >> t) & 1) ? x : fsub(fe_one(), x));
    }
    b2[i] = v;
  }
  std::vector<fe> lambda = aggregate_weights(N, b2.data());
  OpenBufs ob;
  ob.pool = &ctx->pools["pcs_claim:" + std::to_string(N) + ":" + std::to_string(pcs->sc.M) + ":" +
                        std::to_string(pcs->Bs) + ":" + std::to_string(nb)];
  fe *dr = ob.alloc<fe>(nr), *dl = ob.alloc<fe>(N), *brow = ob.alloc<fe>(32), *bcol = ob.alloc<fe>(pcs->Bs),
     *dK = ob.alloc<fe>(1);
  GBZ_CUDA(cudaMemcpyAsync(dr, hr.data(), 16ull * nr, cudaMemcpyHostToDevice, s));
  GBZ_CUDA(cudaMemcpyAsync(dl, lambda.data(), 16ull * N, cudaMemcpyHostToDevice, s));
  // the weights of v[32 j + i]: beta over (r1: 5, r2: log2 Bs) = brow[i] bcol[j]
  beta_launch(dr + lk, 5, brow, s);
  beta_launch(dr + lk + 5, logBs, bcol, s);
  const int nblk = (int)std::min<uint64_t>(64, (pcs->Bs + kRedThreads - 1) / kRedThreads);
  fe *partial = ob.alloc<fe>((uint64_t)N * nblk);
  if (nb - 1 > 32) throw ArgError("pcs: F_ip over more than 32 rows");
  k_fip_partial<<<dim3(nblk, N), kRedThreads, 0, s>>>(pcs->cd, (uint64_t)nb * pcs->Bs, nb - 1, pcs->Bs, brow, bcol,
                                                       partial);
  k_fip_combine<<<1, kPcsMaxParties, 0, s>>>(partial, nblk, N, dl, dK);
  GBZ_CUDA(cudaGetLastError());
  if (mem == GBZ_MEM_DEVICE) GBZ_CUDA(cudaMemcpyAsync(K, dK, 16, cudaMemcpyDeviceToDevice, s));
  else GBZ_CUDA(cudaMemcpyAsync(K, dK, 16, cudaMemcpyDeviceToHost, s));
  GBZ_CUDA(cudaStreamSynchronize(s));
  API_END(ctx)
}

gbz_status gbz_pcs_claim_piop(gbz_ctx *ctx, const gbz_pcs *pcs, const uint64_t *b1, int nb1, const uint64_t *b2,
                              uint64_t nb2, const uint64_t *b3, int nb3, uint64_t *K, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(pcs, "pcs");
  need(b1, "b1");
  need(b2, "b2");
  need(b3, "b3");
  need(K, "K");
  if (pcs->device != ctx->device) throw ArgError("pcs: committed on another device");
  const int N = pcs->sc.N, nb = pcs->batches;
  const uint64_t Bs = pcs->Bs, q0 = (uint64_t)pcs->sc.queries[0];
  if (nb1 < 0) throw ArgError("pcs: b1 length");
  if (nb2 != Bs) throw ArgError("pcs: b2 must have the row length's entries");
  if (nb3 != N / 4) throw ArgError("pcs: b3 must have N/4 entries");
  if (q0 >= Bs) throw ArgError("pcs: _queries[0] must be below the row length");
  cudaStream_t s = ctx->stream;
  const cudaMemcpyKind kin = mem == GBZ_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  std::vector<fe> hb3(N / 4);
  GBZ_CUDA(cudaMemcpyAsync(hb3.data(), b3, 16ull * (N / 4),
                           mem == GBZ_MEM_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost, s));
  GBZ_CUDA(cudaStreamSynchronize(s));
  // F_ip's party weights (MPI_utils.cpp:514-527) from b3, as for a point
  std::vector<fe> lambda = aggregate_weights(N, hb3.data());
  OpenBufs ob;
  ob.pool = &ctx->pools["pcs_claim_piop:" + std::to_string(N) + ":" + std::to_string(pcs->sc.M) + ":" +
                        std::to_string(Bs) + ":" + std::to_string(nb)];
  fe *d1 = ob.alloc<fe>(32), *d2 = ob.alloc<fe>(Bs), *dl = ob.alloc<fe>(N), *dK = ob.alloc<fe>(1);
  const int n1 = std::min(nb1, 32);
  GBZ_CUDA(cudaMemsetAsync(d1, 0, 16 * 32, s));
  if (n1 > 0) GBZ_CUDA(cudaMemcpyAsync(d1, b1, 16ull * n1, kin, s));
  GBZ_CUDA(cudaMemcpyAsync(d2, b2, 16 * Bs, kin, s));
  if (q0) GBZ_CUDA(cudaMemsetAsync(d2 + (Bs - q0), 0, 16 * q0, s));
  GBZ_CUDA(cudaMemcpyAsync(dl, lambda.data(), 16ull * N, cudaMemcpyHostToDevice, s));
  const int nblk = (int)std::min<uint64_t>(64, (Bs + kRedThreads - 1) / kRedThreads);
  fe *partial = ob.alloc<fe>((uint64_t)N * nblk);
  if (nb - 1 > 32) throw ArgError("pcs: F_ip over more than 32 rows");
  k_fip_partial<<<dim3(nblk, N), kRedThreads, 0, s>>>(pcs->cd, (uint64_t)nb * Bs, nb - 1, Bs, d1, d2, partial);
  k_fip_combine<<<1, kPcsMaxParties, 0, s>>>(partial, nblk, N, dl, dK);
  GBZ_CUDA(cudaGetLastError());
  if (mem == GBZ_MEM_DEVICE) GBZ_CUDA(cudaMemcpyAsync(K, dK, 16, cudaMemcpyDeviceToDevice, s));
  else GBZ_CUDA(cudaMemcpyAsync(K, dK, 16, cudaMemcpyDeviceToHost, s));
  GBZ_CUDA(cudaStreamSynchronize(s));
  API_END(ctx)
}

static gbz_status pcs_open_impl(gbz_ctx *ctx, gbz_pcs *pcs, const uint64_t *r, int nr, const uint64_t *K,
                                uint64_t *fs, bool full, gbz_prng *prng, uint32_t *flags, uint8_t *transcript,
                                uint64_t capacity, int mem, const PiopIn *pi = nullptr) {
  API_BEGIN(ctx)
  check_mem(mem);
  if (full) need(prng, "prng");
  need(pcs, "pcs");
  if (!pi) need(r, "r");
  need(K, "K");
  need(fs, "fs");
  need(transcript, "transcript");
  if (pcs->device != ctx->device) throw ArgError("pcs: committed on another device");
  const PcsSchedule &sc = pcs->sc;
  const int N = sc.N, logN = ilog2(N), nb = pcs->batches;
  const uint64_t Bs = pcs->Bs, L = pcs->L;
  const int lk = ilog2(N / 4), logBs = ilog2(Bs);
  if (pi) {
    need(pi->b1, "b1");
    need(pi->b2, "b2");
    need(pi->b3, "b3");
    need(pi->lag, "lagrange");
    need(pi->loglag, "log_lengths");
    if (pi->nb1 < 0) throw ArgError("pcs: b1 length");
    if (pi->nb2 != Bs) throw ArgError("pcs: b2 must have the row length's entries");
    if (pi->nb3 != N / 4) throw ArgError("pcs: b3 must have N/4 entries");
    if ((uint64_t)sc.queries[0] >= Bs) throw ArgError("pcs: _queries[0] must be below the row length");
    nr = 0;
  } else if (nr != lk + 5 + logBs) {
    throw ArgError("pcs: the point must have log2(N/4) + 5 + log2(row length) entries");
  }
  PcsLayout lay;
  const OpenOffs off = open_layout(*pcs, lay);
  const uint64_t tail_base = lay.bytes;
  LeaderInputs lead = leader_shape(*pcs, pi);
  std::vector<DrawOp> script;
  uint64_t arena_len = 0;
  if (full) tail_layout(*pcs, lay, &script, &arena_len, pi);
  if (capacity < lay.bytes)
    throw ArgError(full ? "pcs: transcript capacity below gbz_pcs_open_full_bytes"
                        : "pcs: transcript capacity below gbz_pcs_info's open_transcript_bytes");
  cudaStream_t s = ctx->stream;
  // an opening makes the same allocations for the same shape: the
  // context's pool for this shape serves them after the first
  OpenBufs ob;
  {
    std::string key = "pcs_open" + std::to_string((int)full) + (pi ? "p" + std::to_string(pi->nlag) : std::string()) +
                      ":" + std::to_string(mem) + ":" + std::to_string(N) +
                      ":" + std::to_string(pcs->sc.M) + ":" + std::to_string(sc.rounds);
    for (int i = 0; i < sc.rounds; i++) key += ":" + std::to_string(sc.rate0[i]) + "/" + std::to_string(sc.rate1[i]);
    ob.pool = &ctx->pools[key];
  }
  uint8_t *tr = mem == GBZ_MEM_DEVICE ? transcript : ob.alloc<uint8_t>(lay.bytes);
  // headers
  Hdr *dh = ob.alloc<Hdr>(lay.hdr.size());
  GBZ_CUDA(cudaMemcpyAsync(dh, lay.hdr.data(), sizeof(Hdr) * lay.hdr.size(), cudaMemcpyHostToDevice, s));
  k_headers<<<grid(lay.hdr.size()), 256, 0, s>>>(dh, (int)lay.hdr.size(), tr);
  GBZ_CUDA(cudaGetLastError());
  // The leader's draws depend on the generator alone: the script draws them
  // on the side stream while the parties' rounds run.
  ProofState *pst = nullptr;
  uint32_t *dfl = nullptr;
  LeaderDraws ldraws;
  const SideStream *side = nullptr;
  if (full) {
    glibc_prng g0;
    static_assert(sizeof(glibc_prng) == sizeof(gbz_prng), "generator layouts");
    std::memcpy(&g0, prng, sizeof g0);
    pst = ob.alloc<ProofState>(1);
    dfl = ob.alloc<uint32_t>(1);
    ldraws.arena = ob.alloc<fe>(std::max<uint64_t>(arena_len, 1));
    ldraws.after_walk = ob.alloc<glibc_prng>(1);
    ldraws.final_state = ob.alloc<glibc_prng>(1);
    DrawOp *dops = ob.alloc<DrawOp>(script.size());
    GBZ_CUDA(cudaMemcpyAsync(dops, script.data(), sizeof(DrawOp) * script.size(), cudaMemcpyHostToDevice, s));
    leader_tail_init(pst, g0, dfl, s);
    side = &ctx->side_stream();
    GBZ_CUDA(cudaEventRecord(side->fork, s));
    GBZ_CUDA(cudaStreamWaitEvent(side->stream, side->fork, 0));
    leader_draws_launch(g0, dops, (int)script.size(), ldraws, tr + tail_base, pst, side->stream);
    GBZ_CUDA(cudaEventRecord(side->join, side->stream));
  }
  // point and constants
  std::vector<fe> hr(nr);
  for (int i = 0; i < nr; i++) {
    if (mem == GBZ_MEM_DEVICE) break;
    hr[i] = fe_make(r[2 * i], r[2 * i + 1]);
  }
  fe *dr = ob.alloc<fe>(std::max(nr, 1));
  if (nr)
    GBZ_CUDA(cudaMemcpyAsync(dr, mem == GBZ_MEM_DEVICE ? (const void *)r : (const void *)hr.data(), 16ull * nr,
                             mem == GBZ_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  fe hK, hfs;
  if (mem == GBZ_MEM_DEVICE) {
    uint64_t t[4];
    GBZ_CUDA(cudaMemcpyAsync(t, K, 16, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaMemcpyAsync(t + 2, fs, 16, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaStreamSynchronize(s));
    hK = fe_make(t[0], t[1]);
    hfs = fe_make(t[2], t[3]);
  } else {
    hK = fe_make(K[0], K[1]);
    hfs = fe_make(fs[0], fs[1]);
  }
  PcsDev *st = ob.alloc<PcsDev>(1);
  k_init<<<1, 1, 0, s>>>(st, hfs, hK);
  GBZ_CUDA(cudaGetLastError());
  std::vector<fe> mu = shamir_share_matrix(N), scale((size_t)N * N);
  for (int a = 0; a < N; a++)
    for (int p = 0; p < N; p++) scale[(size_t)a * N + p] = host_tensor_scale((uint32_t)a, N / 2, p);
  // pcs_sumcheck_aggr (MPI_utils.cpp:362-371) sums the even entries of the
  // unpacked shares, E[2j] for j < N/2: one fixed linear form of the N messages
  std::vector<fe> g(N, fe_zero());
  for (int j = 0; j < N / 2; j++) g[2 * j] = fe_one();
  std::vector<fe> lambda = aggregate_weights_even(N, g);
  fe *dmu = ob.alloc<fe>(mu.size()), *dscale = ob.alloc<fe>(scale.size()), *dlam = ob.alloc<fe>(N);
  GBZ_CUDA(cudaMemcpyAsync(dmu, mu.data(), 16 * mu.size(), cudaMemcpyHostToDevice, s));
  GBZ_CUDA(cudaMemcpyAsync(dscale, scale.data(), 16 * scale.size(), cudaMemcpyHostToDevice, s));
  GBZ_CUDA(cudaMemcpyAsync(dlam, lambda.data(), 16ull * N, cudaMemcpyHostToDevice, s));

  // betas of the point: r3 (log2 N/4), r1 (5), r2 (log2 Bs) (coPCS.cpp:1319-1325)
  // or, in the PIOP mode, the input vectors with b2's last _queries[0]
  // entries zeroed (:1327-1335) and b1 cut to the batches (:1349)
  fe *b1 = ob.alloc<fe>(32), *b2 = ob.alloc<fe>(Bs), *b3 = ob.alloc<fe>(std::max(1, N / 4)), *b3p = ob.alloc<fe>(N);
  fe *dlag = nullptr;
  if (pi) {
    const cudaMemcpyKind kin = mem == GBZ_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const int n1 = std::min(pi->nb1, std::min(nb - 1, 32));
    const uint64_t q0 = (uint64_t)sc.queries[0];
    GBZ_CUDA(cudaMemsetAsync(b1, 0, 16 * 32, s));
    if (n1 > 0) GBZ_CUDA(cudaMemcpyAsync(b1, pi->b1, 16ull * n1, kin, s));
    GBZ_CUDA(cudaMemcpyAsync(b2, pi->b2, 16 * Bs, kin, s));
    if (q0) GBZ_CUDA(cudaMemsetAsync(b2 + (Bs - q0), 0, 16 * q0, s));
    GBZ_CUDA(cudaMemcpyAsync(b3, pi->b3, 16ull * (N / 4), kin, s));
    uint64_t nl = 0;
    for (int k = 0; k < pi->nlag; k++) nl += 1ull << pi->loglag[k];
    dlag = ob.alloc<fe>(nl);
    GBZ_CUDA(cudaMemcpyAsync(dlag, pi->lag, 16 * nl, kin, s));
  } else {
    beta_launch(dr + lk, 5, b1, s);
    beta_launch(dr + lk + 5, logBs, b2, s);
    if (lk) beta_launch(dr, lk, b3, s);
    else {
      const fe one = fe_one();
      GBZ_CUDA(cudaMemcpyAsync(b3, &one, 16, cudaMemcpyHostToDevice, s));
    }
  }
  k_b3p<<<1, 64, 0, s>>>(b3, N / 4, dmu, N, b3p);
  GBZ_CUDA(cudaGetLastError());
  // row batching (coPCS.cpp:1352-1356) and the transforms of :1359-1366
  fe *Cp = ob.alloc<fe>((uint64_t)N * L), *bcd = ob.alloc<fe>((uint64_t)N * Bs), *cdl = ob.alloc<fe>((uint64_t)N * Bs);
  fe *B = ob.alloc<fe>((uint64_t)N * Bs), *tmp = ob.alloc<fe>(std::max<uint64_t>((uint64_t)N * L, 1ull << 13));
  k_lincomb<<<dim3(grid(Bs), N), 256, 0, s>>>(pcs->cd, (uint64_t)nb * Bs, Bs, nb - 1, Bs, b1, bcd, Bs);
  GBZ_CUDA(cudaGetLastError());
  // C' = sum_i b1[i] Codeword[i] is Encode of the batched data: every
  // codeword row is Encode(Commit_data row) and Encode is linear, so one
  // encode of bcd per party replaces reading the nb - 1 codeword rows
  encode_rows_device(ctx, bcd, N, logBs, sc.rate0[0], sc.log_rate_offset, Cp);
  GBZ_CUDA(cudaMemcpy2DAsync(cdl, 16 * Bs, pcs->cd + (uint64_t)(nb - 1) * Bs, 16ull * nb * Bs, 16 * Bs, N,
                             cudaMemcpyDeviceToDevice, s));
  const NttTables &tB = ctx->tables(logBs);
  ntt_launch(tB, b2, Bs, b2, tmp, false, s);
  ntt_launch_rows(tB, bcd, Bs, Bs, bcd, Bs, N, tmp, true, s);
  ntt_launch_rows(tB, cdl, Bs, Bs, cdl, Bs, N, tmp, true, s);
  const NttTables &tw = ctx->tables(1 + sc.log_rate_offset + logBs);
  k_open_prep<<<dim3(grid(Bs), N), 256, 0, s>>>(bcd, cdl, B, b2, b3p, Bs, tw.lo_fwd, tw.hi_fwd, tw.lo_inv,
                                                 tw.hi_inv);
  GBZ_CUDA(cudaGetLastError());
  // the batching round
  const int nblk = (int)std::min<uint64_t>(64, (Bs + kRedThreads - 1) / kRedThreads);
  fe *partial = ob.alloc<fe>(2ull * N * nblk), *H = ob.alloc<fe>((uint64_t)N * (2 << kPcsMaxLogDeg));
  fe *poly = ob.alloc<fe>(2 << kPcsMaxLogDeg);
  k_first_partial<<<dim3(nblk, N), kRedThreads, 0, s>>>(bcd, cdl, B, Bs, partial);
  k_first_reduce<<<1, 64, 0, s>>>(partial, nblk, N, H, tr, off.pp0);
  aggregate_launch(H, N, 3, dlam, poly, s);
  k_first_verify<<<1, 1, 0, s>>>(st, poly, tr, off.poly0, off.chal0, off.K0);
  k_first_fold<<<dim3(grid(L), N), 256, 0, s>>>(bcd, cdl, B, Cp, pcs->cw + (uint64_t)(nb - 1) * L, (uint64_t)nb * L,
                                                Bs, L, st);
  GBZ_CUDA(cudaGetLastError());
  // batch_commitments_new (coPCS.cpp:1242-1308): the root over C' in columns
  // of _degrees[1] entries depends on the first column's first leaf
  // (C'[0], C'[c], C'[2c], C'[3c], c = L / d1): that leaf hashed
  // log2(d1 / 4) times is the column root, then log2(c) times the party root.
  uint8_t *rts = ob.alloc<uint8_t>(32ull * N), *prev_rts = ob.alloc<uint8_t>(32ull * N);
  int batch_depth = 0;
  {
    const uint64_t c = L / sc.degrees[1];
    k_roots<<<1, 64, 0, s>>>(Cp, L, c, ilog2(sc.degrees[1] / 4) + ilog2(c), N, logN, nullptr, rts, tr, off.broots,
                             off.bleader);
    GBZ_CUDA(cudaGetLastError());
    // the batch tree is the commitment a tensor code would inherit when no
    // concatenated commitment follows it (levels over c column roots)
    GBZ_CUDA(cudaMemcpyAsync(prev_rts, rts, 32ull * N, cudaMemcpyDeviceToDevice, s));
    batch_depth = ilog2(c);
  }
  int32_t *qp = ob.alloc<int32_t>(kPcsMaxQueries), *qpos = ob.alloc<int32_t>(kPcsMaxQueries);
  if (!is_pow2(L) || L > 0xFFFFFFFFull) throw ArgError("pcs: codeword length must be a power of two below 2^32");
  k_indexes<<<1, 256, 0, s>>>(st, sc.queries[0], N, (uint32_t)L, qp, qpos, tr, off.bqueries);
  GBZ_CUDA(cudaGetLastError());

  // the rounds (coPCS.cpp:1452-1600)
  fe *Ld = ob.alloc<fe>(1 << kPcsMaxLogDeg), *vscr = ob.alloc<fe>(4 << kPcsMaxLogDeg), *y = ob.alloc<fe>(kPcsMaxQueries);
  uint32_t *q3 = ob.alloc<uint32_t>(kPcsMaxQueries);
  fe *wts = ob.alloc<fe>((uint64_t)N * kPcsMaxQueries);
  uint64_t n = Bs, cpl = L;
  int prev_depth = batch_depth;
  // every party's RS fold of a codeword of length len by 2^logd with the
  // current weights Ld (k_fold_q)
  auto rs_fold = [&](const fe *cw, uint64_t len, int logd, fe *out, uint64_t ostride) {
    fe *iQ = ob.alloc<fe>(len), *t2 = ob.alloc<fe>(len);
    GBZ_CUDA(cudaMemsetAsync(iQ, 0, 16 * len, s));
    GBZ_CUDA(cudaMemcpyAsync(iQ, Ld, 16ull << logd, cudaMemcpyDeviceToDevice, s));
    ntt_launch(ctx->tables(ilog2(len)), iQ, len, iQ, t2, true, s);
    const fe scale = fe_make(len >> logd, 0);
    k_fold_q<<<dim3(grid(len >> logd), N), 256, 0, s>>>(cw, len, logd, iQ, scale, out, ostride);
    GBZ_CUDA(cudaGetLastError());
  };
  const int nrounds = sc.rounds - 1;
  for (int i = 0; i < nrounds; i++) {
    const RoundOffs &ro = off.r[i];
    const int d = sc.degrees[i + 1], logd = ilog2((uint64_t)d), D = 2 * d;
    const uint64_t blocks = (uint64_t)N * n / d;
    // pcs_sumcheck_phase1 (coPCS.cpp:547-566): every party's blocks in one
    // batched transform, the products summed per party
    const NttTables &td = ctx->tables(logd), &tD = ctx->tables(logd + 1);
    fe *e1 = ob.alloc<fe>(blocks * D), *e2 = ob.alloc<fe>(blocks * D), *coef = ob.alloc<fe>((uint64_t)N * n);
    ntt_batched(td, bcd, d, (uint32_t)d, coef, blocks, true, s);
    ntt_batched(tD, coef, d, (uint32_t)d, e1, blocks, false, s);
    ntt_batched(td, B, d, (uint32_t)d, coef, blocks, true, s);
    ntt_batched(tD, coef, d, (uint32_t)d, e2, blocks, false, s);
    const uint64_t pblocks = n / d;
    const int lanes = D >= 256 ? 1 : 256 / D;
    const int per_cta = (int)std::max<uint64_t>((uint64_t)lanes, (pblocks + 607) / 608);
    fe *cpart = ob.alloc<fe>((uint64_t)N * D * cophase1_parts(pblocks, per_cta));
    cophase1_reduce_launch(e1, e2, nullptr, nullptr, nullptr, pblocks, logd + 1, per_cta, cpart, H, s, N);
    k_put_party<<<dim3(grid(D), N), 256, 0, s>>>(H, D, N, tr, ro.pp, 16ull * D);
    aggregate_launch(H, N, D, dlam, poly, s);
    k_round_verify<<<1, 256, 0, s>>>(st, poly, logd, finv(root_of_unity(logd + 1)), finv(fe_make(2ull << logd, 0)),
                                     finv(fe_make(1ull << logd, 0)), Ld, vscr, tr, ro.poly, ro.chal);
    GBZ_CUDA(cudaGetLastError());
    // pcs_sumcheck_phase2 (coPCS.cpp:571-587)
    cophase2_launch(bcd, (uint64_t)N * n, Ld, logd, coef, s);
    GBZ_CUDA(cudaMemcpyAsync(bcd, coef, 16ull * N * n / d, cudaMemcpyDeviceToDevice, s));
    cophase2_launch(B, (uint64_t)N * n, Ld, logd, coef, s);
    GBZ_CUDA(cudaMemcpyAsync(B, coef, 16ull * N * n / d, cudaMemcpyDeviceToDevice, s));
    n /= d;
    const bool last = i == nrounds - 1;
    fe *Cpn, *fold;
    uint64_t cpl_new;
    const uint64_t seg_n = cpl / d;
    if (!last) {
      // encode_concatenated (coPCS.cpp:653-677) and commit_concatenated (:679-738)
      const int r0 = sc.rate0[i + 2], r1 = sc.rate1[i + 2], d2 = sc.degrees[i + 2];
      cpl_new = n * r0;
      const uint64_t rows = cpl_new / d2, Dc = (uint64_t)d2 * r1;
      if (ilog2(cpl_new) > kMaxNttLogN || Dc > (1u << 13) || (uint64_t)d2 > cpl_new)
        throw ArgError("pcs: concatenated code shape out of range");
      Cpn = ob.alloc<fe>((uint64_t)N * cpl_new);
      fe *Cn = ob.alloc<fe>((uint64_t)N * rows * Dc);
      fe *tmp2 = ob.alloc<fe>((uint64_t)N * cpl_new);
      ntt_launch_rows(ctx->tables(ilog2(cpl_new)), bcd, n, n, Cpn, cpl_new, N, tmp2, false, s);
      const NttTables &tc = ctx->tables(ilog2(Dc));
      for (int p = 0; p < N; p++)
        ntt_batched_strided(tc, Cpn + (uint64_t)p * cpl_new, rows, (uint32_t)d2, Cn + (uint64_t)p * rows * Dc, rows,
                            false, s);
      const uint64_t clen = rows * Dc;
      k_roots<<<1, 64, 0, s>>>(Cn, clen, 1, ilog2(clen / 4), N, logN, nullptr, rts, tr, ro.roots, ro.leader);
      GBZ_CUDA(cudaGetLastError());
      GBZ_CUDA(cudaMemcpyAsync(prev_rts, rts, 32ull * N, cudaMemcpyDeviceToDevice, s));
      prev_depth = ilog2(clen / 4);
      fold = ob.alloc<fe>((uint64_t)N * seg_n);
      rs_fold(Cp, cpl, logd, fold, seg_n);
    } else {
      // RS_multifold5 + commit_tensorcode (coPCS.cpp:1566-1570, 893-919)
      cpl_new = cpl / d;
      Cpn = ob.alloc<fe>((uint64_t)N * cpl_new);
      rs_fold(Cp, cpl, logd, Cpn, cpl_new);
      fold = Cpn;
      // commit_tensorcode hands MT_commit_Blake the previous commitment's
      // levels; MT_commit_Blake resizes only an empty levels vector
      // (merkle_tree.cpp:205-208), so over a shallower tree the old top level
      // stays and the root it reports is the previous root.
      if (cpl_new < 4) throw ArgError("pcs: the tensor codeword is shorter than one leaf");
      const int depth = ilog2(cpl_new / 4);
      // a deeper new tree than the reused levels vector holds is undefined
      // behaviour in the reference (create_tree_blake writes past its end)
      if (depth > prev_depth) throw ArgError("pcs: tensor code deeper than the previous commitment");
      const bool stale = prev_depth > depth;
      k_roots<<<1, 64, 0, s>>>(Cpn, cpl_new, 1, depth, N, logN, stale ? prev_rts : nullptr, rts, tr, ro.roots,
                               ro.leader);
      GBZ_CUDA(cudaGetLastError());
    }
    // delegate_checks (coPCS.cpp:740-891)
    const int l = sc.queries[i + 1];
    if (!is_pow2(seg_n)) throw ArgError("pcs: segment count must be a power of two");
    k_indexes<<<1, 256, 0, s>>>(st, l, N, (uint32_t)seg_n, qp, qpos, tr, ro.queries);
    LeaderRound &lr = lead.rounds[i];
    lr.d = d;
    lr.l = l;
    lr.n = cpl;
    lr.C0 = i ? (uint64_t)sc.degrees[i + 1] * sc.rate1[i + 1] : 0;
    lr.rate_next = i + 2 < sc.rounds ? sc.rate0[i + 2] : 0;
    lr.rate_cur = sc.rate0[i + 1];
    fe *seg_copy = nullptr;
    if (full) {
      fe *Lc = ob.alloc<fe>(d), *yc = ob.alloc<fe>(l);
      int32_t *qpc = ob.alloc<int32_t>(l), *qposc = ob.alloc<int32_t>(l);
      if (i) seg_copy = ob.alloc<fe>((uint64_t)l * d);
      lr.L = Lc;
      lr.y = yc;
      lr.qp = qpc;
      lr.qpos = qposc;
      lr.seg = seg_copy;
    }
    k_gather<<<grid((uint64_t)l * d), 256, 0, s>>>(Cp, cpl, seg_n, d, fold, seg_n, qp, qpos, l, y, tr, ro.y, ro.seg,
                                                   seg_copy);
    GBZ_CUDA(cudaGetLastError());
    if (full) {
      GBZ_CUDA(cudaMemcpyAsync((void *)lr.L, Ld, 16ull * d, cudaMemcpyDeviceToDevice, s));
      GBZ_CUDA(cudaMemcpyAsync((void *)lr.y, y, 16ull * l, cudaMemcpyDeviceToDevice, s));
      GBZ_CUDA(cudaMemcpyAsync((void *)lr.qp, qp, 4ull * l, cudaMemcpyDeviceToDevice, s));
      GBZ_CUDA(cudaMemcpyAsync((void *)lr.qpos, qpos, 4ull * l, cudaMemcpyDeviceToDevice, s));
    }
    if (!last) {
      k_check_y<<<grid(l), 256, 0, s>>>(Cpn, cpl_new, (uint32_t)sc.rate0[i + 2], (uint32_t)sc.rate0[i + 1], qp, qpos,
                                        y, l, st);
      GBZ_CUDA(cudaGetLastError());
    }
    k_s_update<<<1, 256, 0, s>>>(st, y, l, last ? 0 : 1, tr, ro.s, ro.K);
    GBZ_CUDA(cudaGetLastError());
    if (full) {
      fe *sc_ = ob.alloc<fe>(1);
      GBZ_CUDA(cudaMemcpyAsync(sc_, &st->s, 16, cudaMemcpyDeviceToDevice, s));
      lr.s = sc_;
    }
    if (!last) {
      // pcs_sumcheck_phase3 (coPCS.cpp:634-648) with the scaled queries
      const int logw = ilog2((uint64_t)sc.rate0[i + 2] * n);
      const uint64_t W = 1ull << logw;
      if (logw > kMaxNttLogN) throw ArgError("pcs: phase-3 transform longer than 2^26");
      fe *V = ob.alloc<fe>((uint64_t)N * W), *T = ob.alloc<fe>((uint64_t)N * W);
      fe *tmp3 = logw > 13 ? ob.alloc<fe>((uint64_t)N * W) : nullptr;
      GBZ_CUDA(cudaMemsetAsync(V, 0, 16ull * N * W, s));
      k_phase3_prep<<<grid(l), 256, 0, s>>>(st, qp, qpos, l, (uint32_t)sc.rate0[i + 2], (uint32_t)sc.rate0[i + 1],
                                             logw, dscale, N, q3, wts);
      k_phase3_scatter<<<dim3(grid(l), N), 256, 0, s>>>(q3, wts, l, W, V);
      GBZ_CUDA(cudaGetLastError());
      ntt_launch_rows(ctx->tables(logw), V, W, W, T, W, N, tmp3, false, s);
      k_phase3_add<<<dim3(grid(n), N), 256, 0, s>>>(B, n, T, W);
      GBZ_CUDA(cudaGetLastError());
    }
    Cp = Cpn;
    cpl = cpl_new;
  }
  // send_pcs_data: every party's data, B and C'
  {
    const uint64_t per = 2 * n + cpl;
    k_put_party<<<dim3(grid(n), N), 256, 0, s>>>(bcd, n, N, tr, off.final_, 16 * per);
    k_put_party<<<dim3(grid(n), N), 256, 0, s>>>(B, n, N, tr, off.final_ + 16 * n, 16 * per);
    k_put_party<<<dim3(grid(cpl), N), 256, 0, s>>>(Cp, cpl, N, tr, off.final_ + 32 * n, 16 * per);
    GBZ_CUDA(cudaGetLastError());
  }
  // the leader's delegation proofs, final checks and WHIR opening
  if (full) {
    lead.bcd = bcd;
    lead.B = B;
    lead.Cp = Cp;
    lead.K = &st->K;
    lead.r_first = &st->r_first;
    lead.b2 = b2;
    lead.b3 = b3;
    lead.r2 = pi ? nullptr : dr + lk + 5;
    if (pi) {
      lead.lag = dlag;
      const uint64_t md = lead.max_delegation;
      for (int c = 0; c < 2 && pi->slots; c++) {
        const gbz_whir_slot &u = pi->slots[c];
        WhirSlotDev &o = lead.slot[c];
        auto place = [&](void *user, uint64_t bytes) -> void * {
          if (!user) return nullptr;
          return mem == GBZ_MEM_DEVICE ? user : (void *)ob.alloc<uint8_t>(bytes);
        };
        o.arr = (fe *)place(u.arr, 16 * md);
        o.cw = (fe *)place(u.codeword, 64 * md);
        o.betas = (fe *)place(u.betas, 16 * md);
        o.claim = (fe *)place(u.claim, 16);
        o.root = (uint8_t *)place(u.root, 32);
      }
    }
    // unpack_secret_share(., N/2, N) (MPI_utils.cpp:2769-2785): output j is
    // entry 2j of the unpacked shares, a fixed linear form of the N shares
    std::vector<fe> U((size_t)(N / 2) * N);
    for (int j = 0; j < N / 2; j++) {
      std::vector<fe> gj(N, fe_zero());
      gj[2 * j] = fe_one();
      const std::vector<fe> w = aggregate_weights_even(N, gj);
      for (int p = 0; p < N; p++) U[(size_t)j * N + p] = w[p];
    }
    fe *dU = ob.alloc<fe>(U.size());
    GBZ_CUDA(cudaMemcpyAsync(dU, U.data(), 16 * U.size(), cudaMemcpyHostToDevice, s));
    lead.unpack = dU;
    GBZ_CUDA(cudaStreamWaitEvent(s, side->join, 0));
    LeaderResources LR;
    LR.s = s;
    LR.alloc = [&ob](uint64_t bytes) -> void * { return ob.alloc<uint8_t>(bytes); };
    LR.tables = [ctx](int lg) -> NttTables & { return ctx->tables(lg); };
    Layout tl;
    uint64_t used = 0;
    leader_tail(LR, lead, pst, dfl, tr + tail_base, tl, nullptr, &used, &ldraws);
    if (used != arena_len) throw ArgError("pcs: leader draw count mismatch");
    if (tail_base + tl.len != lay.bytes) throw ArgError("pcs: leader transcript layout mismatch");
  }
  // the chain state out, the flags checked
  PcsDev hst;
  uint32_t hfl = 0;
  glibc_prng hg{};
  GBZ_CUDA(cudaMemcpyAsync(&hst, st, sizeof(PcsDev), cudaMemcpyDeviceToHost, s));
  if (full) {
    GBZ_CUDA(cudaMemcpyAsync(&hfl, dfl, 4, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaMemcpyAsync(&hg, ldraws.final_state, sizeof hg, cudaMemcpyDeviceToHost, s));
  }
  if (mem == GBZ_MEM_HOST) GBZ_CUDA(cudaMemcpyAsync(transcript, tr, lay.bytes, cudaMemcpyDeviceToHost, s));
  if (pi && pi->slots && mem == GBZ_MEM_HOST) {
    const uint64_t md = lead.max_delegation;
    for (int c = 0; c < 2; c++) {
      const gbz_whir_slot &u = pi->slots[c];
      const WhirSlotDev &o = lead.slot[c];
      if (u.arr) GBZ_CUDA(cudaMemcpyAsync(u.arr, o.arr, 16 * md, cudaMemcpyDeviceToHost, s));
      if (u.codeword) GBZ_CUDA(cudaMemcpyAsync(u.codeword, o.cw, 64 * md, cudaMemcpyDeviceToHost, s));
      if (u.betas) GBZ_CUDA(cudaMemcpyAsync(u.betas, o.betas, 16 * md, cudaMemcpyDeviceToHost, s));
      if (u.claim) GBZ_CUDA(cudaMemcpyAsync(u.claim, o.claim, 16, cudaMemcpyDeviceToHost, s));
      if (u.root) GBZ_CUDA(cudaMemcpyAsync(u.root, o.root, 32, cudaMemcpyDeviceToHost, s));
    }
  }
  GBZ_CUDA(cudaStreamSynchronize(s));
  if (mem == GBZ_MEM_HOST) {
    fs[0] = hst.fs.re;
    fs[1] = hst.fs.im;
  } else {
    GBZ_CUDA(cudaMemcpy(fs, &hst.fs, 16, cudaMemcpyHostToDevice));
  }
  if (full) {
    std::memcpy(prng, &hg, sizeof hg);
    if (flags) *flags = hfl;
  }
  if (hst.error) return fail(ctx, GBZ_ECHECK, hst.error & 1 ? "pcs: a round message does not match the claim"
                                                            : "pcs: a delegate check failed");
  if (hfl & LF_FATAL) return fail(ctx, GBZ_ECHECK, "pcs: a check of the leader's delegation or final opening failed");
  API_END(ctx)
}

gbz_status gbz_pcs_open(gbz_ctx *ctx, gbz_pcs *pcs, const uint64_t *r, int nr, const uint64_t *K, uint64_t *fs,
                        uint8_t *transcript, uint64_t capacity, int mem) {
  return pcs_open_impl(ctx, pcs, r, nr, K, fs, false, nullptr, nullptr, transcript, capacity, mem);
}

gbz_status gbz_pcs_open_full(gbz_ctx *ctx, gbz_pcs *pcs, const uint64_t *r, int nr, const uint64_t *K, uint64_t *fs,
                             gbz_prng *prng, uint32_t *flags, uint8_t *transcript, uint64_t capacity, int mem) {
  return pcs_open_impl(ctx, pcs, r, nr, K, fs, true, prng, flags, transcript, capacity, mem);
}

gbz_status gbz_pcs_open_piop(gbz_ctx *ctx, gbz_pcs *pcs, const uint64_t *b1, int nb1, const uint64_t *b2,
                             uint64_t nb2, const uint64_t *b3, int nb3, const uint64_t *lagrange,
                             const int *log_lengths, int nlag, const uint64_t *K, uint64_t *fs, gbz_prng *prng,
                             uint32_t *flags, gbz_whir_slot *slots, uint8_t *transcript, uint64_t capacity, int mem) {
  PiopIn pi;
  pi.b1 = b1;
  pi.nb1 = nb1;
  pi.b2 = b2;
  pi.nb2 = nb2;
  pi.b3 = b3;
  pi.nb3 = nb3;
  pi.lag = lagrange;
  pi.loglag = log_lengths;
  pi.nlag = nlag;
  pi.slots = slots;
  if (!log_lengths || nlag < 1 || nlag > 8) return fail(ctx, GBZ_EINVAL, "pcs: 1..8 Lagrange factors with their log2 lengths");
  return pcs_open_impl(ctx, pcs, nullptr, 0, K, fs, true, prng, flags, transcript, capacity, mem, &pi);
}

gbz_status gbz_pcs_open_piop_bytes(const gbz_pcs *pcs, const int *log_lengths, int nlag, uint64_t *bytes,
                                   uint64_t *slot_len) {
  if (!pcs || !bytes || !log_lengths || nlag < 1 || nlag > 8) return GBZ_EINVAL;
  try {
    PiopIn pi;
    pi.loglag = log_lengths;
    pi.nlag = nlag;
    PcsLayout lay;
    open_layout(*pcs, lay);
    tail_layout(*pcs, lay, nullptr, nullptr, &pi);
    *bytes = lay.bytes;
    if (slot_len) *slot_len = leader_shape(*pcs).max_delegation;
  } catch (const ArgError &) {
    return GBZ_EINVAL;
  }
  return GBZ_OK;
}

gbz_status gbz_pcs_open_full_bytes(const gbz_pcs *pcs, uint64_t *bytes) {
  if (!pcs || !bytes) return GBZ_EINVAL;
  try {
    PcsLayout lay;
    open_layout(*pcs, lay);
    tail_layout(*pcs, lay);
    *bytes = lay.bytes;
  } catch (const ArgError &) {
    return GBZ_EINVAL;
  }
  return GBZ_OK;
}

gbz_status gbz_cosumcheck(gbz_ctx *ctx, int form, int N, uint64_t n, const uint64_t *p1, const uint64_t *p2,
                          const uint64_t *p3, const uint64_t *R, const uint64_t *r1, int nr1, const uint64_t *r2,
                          const uint64_t *K, const uint64_t *K_r, const int *degrees, int ndeg, uint64_t *fs,
                          uint64_t *claims, uint32_t *flags, uint8_t *transcript, uint64_t capacity, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(p1, "p1");
  need(p2, "p2");
  need(R, "R");
  need(K, "K");
  need(K_r, "K_r");
  need(degrees, "degrees");
  need(fs, "fs");
  need(claims, "claims");
  const bool cubic = form == GBZ_SC_CUBIC;
  if (cubic) {
    need(p3, "p3");
    need(r1, "r1");
  }
  if (transcript && capacity < cosumcheck_bytes(form, N, degrees, ndeg))
    throw ArgError("coSumcheck: transcript capacity too small");
  if (N < 4 || !is_pow2((uint64_t)N)) throw ArgError("coSumcheck: N must be a power of two in [4, 64]");
  const int lq = ilog2((uint64_t)(N / 4));
  if (cubic && nr1 < 0) throw ArgError("coSumcheck: r1 must have log2(n) entries");
  // the scalars and points to the host
  std::vector<fe> hr1(cubic ? nr1 : 0), hr2(lq);
  fe hK, hKr, hfs;
  const cudaStream_t s = ctx->stream;
  if (mem == GBZ_MEM_DEVICE) {
    if (cubic && nr1) GBZ_CUDA(cudaMemcpyAsync(hr1.data(), r1, 16ull * nr1, cudaMemcpyDeviceToHost, s));
    if (cubic && lq) GBZ_CUDA(cudaMemcpyAsync(hr2.data(), r2, 16ull * lq, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaMemcpyAsync(&hK, K, 16, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaMemcpyAsync(&hKr, K_r, 16, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaMemcpyAsync(&hfs, fs, 16, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaStreamSynchronize(s));
  } else {
    if (cubic) {
      for (int i = 0; i < nr1; i++) hr1[i] = fe_make(r1[2 * i], r1[2 * i + 1]);
      for (int i = 0; i < lq; i++) hr2[i] = fe_make(r2[2 * i], r2[2 * i + 1]);
    }
    hK = fe_make(K[0], K[1]);
    hKr = fe_make(K_r[0], K_r[1]);
    hfs = fe_make(fs[0], fs[1]);
  }
  const cudaMemcpyKind kin = mem == GBZ_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind ko = mem == GBZ_MEM_DEVICE ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
  const CoscOut res = cosumcheck_run(ctx, form, N, n, (const fe *)p1, (const fe *)p2, (const fe *)p3, (const fe *)R, kin,
                                     hr1.data(), nr1, hr2.data(), hK, hKr, degrees, ndeg, hfs, transcript,
                                     mem == GBZ_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, nullptr);
  GBZ_CUDA(cudaMemcpy(claims, res.claims.data(), 16 * res.claims.size(), ko));
  GBZ_CUDA(cudaMemcpy(fs, &res.fs, 16, ko));
  if (flags) *flags = res.flags;
  API_END(ctx)
}

uint64_t gbz_cosumcheck_transcript_bytes(int form, int N, const int *degrees, int ndeg) {
  return cosumcheck_bytes(form, N, degrees, ndeg);
}

}  // extern "C"
