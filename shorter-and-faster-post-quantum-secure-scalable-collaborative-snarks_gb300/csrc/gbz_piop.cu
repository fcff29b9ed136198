// The R1CS front end's two sumcheck phases for N parties on one device
// (prove_phase1 / prove_phase2, coPIOP.cpp:241-627, as coPIOP_prove runs
// them with one MPI rank per party) and the reduction of the parties' R1CS
// rows they use (_reduce_R1CS_matrixes_multivariate,
// Distributed_Sumcheck.cpp:2283-2350).
//
// Every per-party vector is one party-major device array [party][entry].
// The large steps (the masked extension of vL, vR, vO; the reduction of the
// three matrices' rows; the packed resharing and its segment layout; the
// tensor of the Lagrange vectors; the coSumchecks themselves) run as
// launches over all parties.  The scalars that the reference's leader
// computes between them (Fiat-Shamir draws, the interpolation of the
// parties' y shares, the Lagrange vectors over N/4 and 2 points) are a few
// dozen field operations and are made on the host between launches.
#include <cstring>
#include <string>
#include <vector>

#include "gbz_copcs.cuh"
#include "gbz_ctx.cuh"

using namespace gbz_api;

// The parties' R1CS rows (what pA, pB, pC hold on every rank,
// MPI_utils.cpp:2205-2270): per matrix one CSR over the N x rows rows,
// party p owning rows [p rows, (p + 1) rows); an entry is the column
// (constraint index) of a nonzero, all nonzeros being 1.
struct gbz_r1cs {
  int device = 0;
  int N = 0, logm = 0;
  uint64_t rows = 0;
  uint32_t *ptr[3] = {nullptr, nullptr, nullptr};
  uint32_t *cols[3] = {nullptr, nullptr, nullptr};
  uint64_t nnz[3] = {0, 0, 0};
};

namespace gbz {
namespace {

enum : uint32_t { T_PIOP_DRAWS = 58, T_PIOP_Y = 59, T_PIOP_ABC = 60 };
constexpr int kPiopMaxParties = 64;
constexpr int kPiopMaxRounds = 16;

unsigned nblk(uint64_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------------------ host scalars

// hash_to_field({0}) (Fiat_Shamir.cpp:29-35): one step of the chain.
fe draw(fe &fs) {
  fs = hash_F(fs, fe_zero());
  return fs;
}

// compute_lagrange_coeff(getRootOfUnity(logd), r, 2^logd) (utils.cpp:169-172):
// the inverse transform of (1, r, ..., r^{d-1}); for the few small vectors
// the leader forms (d <= 64).
std::vector<fe> host_lagrange(fe r, int logd) {
  const uint64_t d = 1ull << logd;
  std::vector<fe> pw(d);
  pw[0] = fe_one();
  for (uint64_t j = 1; j < d; j++) pw[j] = fmul(pw[j - 1], r);
  const fe wi = finv(root_of_unity(logd)), dinv = finv(fe_make(d, 0));
  std::vector<fe> out(d);
  fe wk = fe_one();
  for (uint64_t k = 0; k < d; k++) {
    fe acc = fe_zero(), x = fe_one();
    for (uint64_t j = 0; j < d; j++) {
      acc = fadd(acc, fmul(pw[j], x));
      x = fmul(x, wk);
    }
    out[k] = fmul(acc, dinv);
    wk = fmul(wk, wi);
  }
  return out;
}

// Entry 0 of the same vector: d^{-1} sum_j r^j.
fe host_lagrange0(fe r, int logd) {
  const uint64_t d = 1ull << logd;
  fe acc = fe_zero(), x = fe_one();
  for (uint64_t j = 0; j < d; j++) {
    acc = fadd(acc, x);
    x = fmul(x, r);
  }
  return fmul(acc, finv(fe_make(d, 0)));
}

// The first `count` entries of the same vector.
std::vector<fe> host_lagrange_head(fe r, int logd, int count) {
  const uint64_t d = 1ull << logd;
  const fe wi = finv(root_of_unity(logd)), dinv = finv(fe_make(d, 0));
  std::vector<fe> out(count);
  fe wk = fe_one();
  for (int k = 0; k < count; k++) {
    fe acc = fe_zero(), x = fe_one(), rp = fe_one();
    for (uint64_t j = 0; j < d; j++) {
      acc = fadd(acc, fmul(rp, x));
      rp = fmul(rp, r);
      x = fmul(x, wk);
    }
    out[k] = fmul(acc, dinv);
    wk = fmul(wk, wi);
  }
  return out;
}

// b[2p + 1] of compute_beta_shares_multivariate (coPIOP.cpp:366-377) and of
// the phases' ip scaling: the N/4 values v zero-padded to N/2, shared as
// compute_secret_shares does: party p's share sum_t mu[p][t] v[t].
std::vector<fe> share_scalars(const std::vector<fe> &v, int N) {
  const std::vector<fe> mu = shamir_share_matrix(N);
  std::vector<fe> out(N, fe_zero());
  for (int p = 0; p < N; p++)
    for (size_t t = 0; t < v.size(); t++) out[p] = fadd(out[p], fmul(mu[(size_t)p * (N / 2) + t], v[t]));
  return out;
}

// ------------------------------------------------------------ kernels

struct Segs {
  int n;
  uint32_t off[kPiopMaxRounds + 1];
};

__global__ void k_one(fe *out) { out[0] = fe_one(); }

// out[j + k na] = b[k] a[j] (the products of _reduce_R1CS_matrixes_multivariate
// and compute_beta_shares_multivariate, Distributed_Sumcheck.cpp:2304-2313,
// coPIOP.cpp:352-363).
__global__ void k_tensor(const fe *a, uint64_t na, const fe *b, uint64_t nb, fe *out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= na * nb) return;
  out[i] = fmul(b[i / na], a[i % na]);
}

// prove_phase1's y and compute_Kr's sums for every party and the leader
// (coPIOP.cpp:263-300, MPI_utils.cpp:3620-3631 with sum, :3370-3414):
// y_p = sum_{i<4} beta_i (rL_i rR_i - rO_i), kr_p = sum over the rounds of
// every fourth entry of the party's share of R1; the leader combines both
// with lambda (unpack, then b2 on the even points).  out: y, K_r, K = y r.
// One CTA, a thread per party.
__global__ void k_piop_y(const fe *masks, const fe *R1, uint64_t rlen, Segs sg, int N, fe b0, fe b1, fe b2, fe b3,
                         const fe *lambda, fe rlast, fe *out, uint8_t *tr, uint64_t off_y) {
  __shared__ fe ys[kPiopMaxParties], ks[kPiopMaxParties];
  const int p = threadIdx.x;
  if (p < N) {
    const fe *m = masks + 12ull * p;
    const fe bt[4] = {b0, b1, b2, b3};
    fe y = fe_zero();
    for (int i = 0; i < 4; i++) y = fadd(y, fmul(bt[i], fsub(fmul(m[i], m[4 + i]), m[8 + i])));
    fe k = fe_zero();
    const fe *r = R1 + (uint64_t)p * rlen;
    for (int i = 0; i < sg.n; i++)
      for (uint32_t j = sg.off[i]; j < sg.off[i + 1]; j += 4) k = fadd(k, r[j]);
    ys[p] = y;
    ks[p] = k;
    put_fe(tr, off_y + 16ull * p, y);
  }
  __syncthreads();
  if (p == 0) {
    fe y = fe_zero(), k = fe_zero();
    for (int q = 0; q < N; q++) {
      y = fadd(y, fmul(lambda[q], ys[q]));
      k = fadd(k, fmul(lambda[q], ks[q]));
    }
    out[0] = y;
    out[1] = k;
    out[2] = fmul(rlast, y);
    put_fe(tr, off_y + 16ull * N, y);
    put_fe(tr, off_y + 16ull * (N + 1), k);
  }
}

// The vectors of the cubic coSumcheck, party-major: vL, vR,
// vO of every party doubled in length, the party's four masks rL, rR, rO at
// the start of the new half, zeros after (coPIOP.cpp:289-298).
__global__ void k_piop_extend(const fe *vL, const fe *vR, const fe *vO, const fe *masks, uint64_t n, int N, fe *out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * n) return;
  const int p = blockIdx.y, v = blockIdx.z;
  const fe *src = v == 0 ? vL : v == 1 ? vR : vO;
  fe x = fe_zero();
  if (i < n)
    x = src[(uint64_t)p * n + i];
  else if (i < n + 4)
    x = masks[12ull * p + 4 * v + (i - n)];
  out[((uint64_t)v * N + p) * 2 * n + i] = x;
}

// Weighted reduction of the R1CS rows: out[g] = w0 X_A(g) + w1 X_B(g) +
// w2 X_C(g), X_M(g) = sum over row g's columns c of beta1[c mod S]
// beta2[c div S] (Distributed_Sumcheck.cpp:2318-2349; a null matrix adds
// nothing).  A thread per row.
struct R1csView {
  const uint32_t *ptr[3];
  const uint32_t *cols[3];
  fe w[3];
};
__global__ void k_r1cs_rows(R1csView m, uint64_t nrows, const fe *beta1, const fe *beta2, int logS, fe scale,
                            fe *out) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nrows) return;
  const uint32_t S1 = (1u << logS) - 1;
  fe acc = fe_zero();
  for (int t = 0; t < 3; t++) {
    if (!m.ptr[t]) continue;
    fe s = fe_zero();
    for (uint32_t e = m.ptr[t][g]; e < m.ptr[t][g + 1]; e++) {
      const uint32_t c = m.cols[t][e];
      s = fadd(s, fmul(beta1[c & S1], beta2[c >> logS]));
    }
    acc = fadd(acc, fmul(m.w[t], s));
  }
  out[g] = fmul(scale, acc);
}

// secret_share_vector (Distributed_Sumcheck.cpp:2352-2400) of every party and
// the alltoall, written straight into prove_phase2's segment layout
// (coPIOP.cpp:470-488): party q shares its vector v_q in groups of N/4 (no
// privacy entries), party p receives its share of every group of every
// party, party by party (len = N rows / (N/4) entries); entry s of that goes
// to segment s div fill at offset s mod fill (fill = seg - mask_l).
__global__ void k_reshare_segments(const fe *v, uint64_t rows, int N, const fe *mu, uint64_t seg, uint64_t fill,
                                   fe *out, uint64_t pstride) {
  const int k = N / 4, kk = N / 2;
  const uint64_t per = rows / k, len = per * N;
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= len) return;
  const int p = blockIdx.y;
  const uint64_t q = s / per, i = s % per;
  const fe *src = v + q * rows + i * k;
  fe acc = fe_zero();
  for (int t = 0; t < k; t++) acc = fadd(acc, fmul(mu[p * kk + t], src[t]));
  out[(uint64_t)p * pstride + (s / fill) * seg + s % fill] = acc;
}

// out[p ostride + off + j] = v[j] scal[p] for j < n.
__global__ void k_scale_parties(const fe *v, uint64_t n, const fe *scal, fe *out, uint64_t ostride, uint64_t off) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int p = blockIdx.y;
  out[(uint64_t)p * ostride + off + j] = fmul(v[j], scal[p]);
}

// The witness side of the second coSumcheck (coPIOP.cpp:449-455, 490): the
// party's witness w, then rL resized to |w| with its first four entries
// a rL + b rR + c rO.
__global__ void k_piop_p1(const fe *w, uint64_t nw, const fe *masks, fe a, fe b, fe c, fe *out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * nw) return;
  const int p = blockIdx.y;
  fe x = fe_zero();
  if (i < nw) {
    x = w[(uint64_t)p * nw + i];
  } else if (i < nw + 4) {
    const fe *m = masks + 12ull * p;
    const uint64_t t = i - nw;
    x = fadd(fadd(fmul(a, m[t]), fmul(b, m[4 + t])), fmul(c, m[8 + t]));
  }
  out[(uint64_t)p * 2 * nw + i] = x;
}

// compute_lagrange_coeff on the device for the reductions' larger vectors:
// powers of r, inverse transform.
void lagrange_dev(gbz_ctx *ctx, fe r, int logd, fe *out, cudaStream_t s) {
  if (logd == 0) {
    k_one<<<1, 1, 0, s>>>(out);
    GBZ_CUDA(cudaGetLastError());
    return;
  }
  const uint64_t d = 1ull << logd;
  powers_launch(r, d, out, s);
  ntt_launch(ctx->tables(logd), out, d, out, nullptr, true, s);
}

// The tensor of the Lagrange vectors of (degree d_i, point r_i) in order
// (the first varies fastest) into out; tmp: two buffers of the result's
// length.
uint64_t lagrange_tensor(gbz_ctx *ctx, const std::vector<int> &degs, const std::vector<fe> &pts, fe *out, fe *t0,
                         fe *t1, cudaStream_t s) {
  uint64_t len = 1;
  fe *cur = t0;
  k_one<<<1, 1, 0, s>>>(cur);
  for (size_t i = 0; i < degs.size(); i++) {
    const int lg = ilog2((uint64_t)degs[i]);
    fe *L = out;  // staged through out, then folded into the other buffer
    lagrange_dev(ctx, pts[i], lg, L, s);
    fe *nxt = cur == t0 ? t1 : t0;
    k_tensor<<<nblk(len * degs[i]), 256, 0, s>>>(cur, len, L, (uint64_t)degs[i], nxt);
    GBZ_CUDA(cudaGetLastError());
    cur = nxt;
    len *= (uint64_t)degs[i];
  }
  GBZ_CUDA(cudaMemcpyAsync(out, cur, 16 * len, cudaMemcpyDeviceToDevice, s));
  return len;
}

// Record headers and small payloads built on the host.
struct HostRecs {
  std::vector<uint8_t> bytes;
  uint64_t add(uint32_t tag, uint32_t count, uint64_t unit) {
    const uint64_t at = bytes.size();
    bytes.resize(at + 8 + unit * count, 0);
    std::memcpy(&bytes[at], &tag, 4);
    std::memcpy(&bytes[at + 4], &count, 4);
    return at + 8;
  }
  void put(uint64_t off, const fe &v) { std::memcpy(&bytes[off], &v, 16); }
};

uint64_t phase1_head_bytes(int N, uint64_t n) {
  const int ln = ilog2(n), lk = ilog2((uint64_t)(N / 4));
  return 8 + 16ull * (ln + lk + 1) + 8 + 16ull * (N + 2);
}

// Copies host values or device words to the caller: kind by mem.
void put_out(gbz_ctx *ctx, void *dst, const void *src, uint64_t bytes, int mem, bool src_on_device) {
  if (!dst || !bytes) return;
  cudaMemcpyKind k;
  if (src_on_device)
    k = mem == GBZ_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  else
    k = mem == GBZ_MEM_DEVICE ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
  GBZ_CUDA(cudaMemcpyAsync(dst, src, bytes, k, ctx->stream));
}

// A caller array on the device: itself, or a pooled copy of host memory.
template <typename T>
const T *in_view(gbz_ctx *ctx, OpenBufs &ob, const T *p, uint64_t count, int mem) {
  if (mem == GBZ_MEM_DEVICE) {
    ob.alloc<uint8_t>(1);  // keeps the pool's allocation sequence the same for both kinds
    return p;
  }
  T *d = ob.alloc<T>(count);
  GBZ_CUDA(cudaMemcpyAsync(d, p, sizeof(T) * count, cudaMemcpyHostToDevice, ctx->stream));
  return d;
}

fe read_fe(gbz_ctx *ctx, const uint64_t *p, int mem) {
  fe v;
  if (mem == GBZ_MEM_DEVICE) {
    GBZ_CUDA(cudaMemcpyAsync(&v, p, 16, cudaMemcpyDeviceToHost, ctx->stream));
    GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  } else {
    v = fe_make(p[0], p[1]);
  }
  return v;
}

std::vector<fe> read_fes(gbz_ctx *ctx, const uint64_t *p, uint64_t count, int mem) {
  std::vector<fe> v(count);
  if (!count) return v;
  if (mem == GBZ_MEM_DEVICE) {
    GBZ_CUDA(cudaMemcpyAsync(v.data(), p, 16 * count, cudaMemcpyDeviceToHost, ctx->stream));
    GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  } else {
    std::memcpy(v.data(), p, 16 * count);
  }
  return v;
}

void check_parties(int N) {
  if (N < 4 || N > kPiopMaxParties || !is_pow2((uint64_t)N))
    throw ArgError("piop: N must be a power of two in [4, 64]");
}

void check_degrees(const int *degrees, int ndeg, const char *what) {
  need(degrees, what);
  if (ndeg < 1 || ndeg > kPiopMaxRounds) throw ArgError(std::string(what) + ": 1..16 rounds");
  for (int i = 0; i < ndeg; i++)
    if (degrees[i] < 1 || degrees[i] > 1024 || !is_pow2((uint64_t)degrees[i]))
      throw ArgError(std::string(what) + ": powers of two up to 1024");
}

// The reduction's tables (Distributed_Sumcheck.cpp:2298-2315): degrees' =
// (N/4, degrees1 without its last), beta1 = the tensor over all of them but
// the last at r[0..], beta2 = the last one's Lagrange vector.  Returns log2
// |beta1| (= the split S of a column).
int reduce_tables(gbz_ctx *ctx, OpenBufs &ob, int N, int logm, const std::vector<fe> &r, const int *degrees1,
                  int ndeg1, fe *&beta1, fe *&beta2, cudaStream_t s) {
  std::vector<int> d(1, N / 4);
  for (int i = 0; i + 1 < ndeg1; i++) d.push_back(degrees1[i]);
  if ((int)r.size() != ndeg1) throw ArgError("r1cs reduce: r must have one entry per degree");
  uint64_t n1 = 1;
  for (int i = 0; i + 1 < ndeg1; i++) n1 *= (uint64_t)d[i];
  const uint64_t n2 = (uint64_t)d[ndeg1 - 1];
  if (n1 * n2 != (1ull << logm)) throw ArgError("r1cs reduce: the degrees must multiply to 2^logm");
  beta1 = ob.alloc<fe>(n1);
  beta2 = ob.alloc<fe>(n2);
  fe *t0 = ob.alloc<fe>(n1), *t1 = ob.alloc<fe>(n1);
  std::vector<int> d1(d.begin(), d.end() - 1);
  std::vector<fe> r1(r.begin(), r.end() - 1);
  if (d1.empty()) {
    k_one<<<1, 1, 0, s>>>(beta1);
  } else {
    lagrange_tensor(ctx, d1, r1, beta1, t0, t1, s);
  }
  lagrange_dev(ctx, r[ndeg1 - 1], ilog2(n2), beta2, s);
  return ilog2(n1);
}

}  // namespace
}  // namespace gbz

using namespace gbz;

extern "C" {

gbz_status gbz_r1cs_create(gbz_ctx *ctx, int N, uint64_t rows, int logm, const uint32_t *const *ptr,
                           const uint32_t *const *cols, const uint64_t *nnz, gbz_r1cs **out) {
  API_BEGIN(ctx)
  need(ptr, "ptr");
  need(cols, "cols");
  need(nnz, "nnz");
  need(out, "out");
  check_parties(N);
  if (rows < 1 || (uint64_t)N * rows >= (1ull << 32)) throw ArgError("r1cs: rows out of range");
  if (logm < 0 || logm > 31) throw ArgError("r1cs: logm out of range");
  const uint64_t total = (uint64_t)N * rows;
  std::unique_ptr<gbz_r1cs> m(new gbz_r1cs);
  m->device = ctx->device;
  m->N = N;
  m->rows = rows;
  m->logm = logm;
  try {
    for (int t = 0; t < 3; t++) {
      need(ptr[t], "ptr[t]");
      if (nnz[t] >= (1ull << 32)) throw ArgError("r1cs: too many entries");
      if (nnz[t]) need(cols[t], "cols[t]");
      if (ptr[t][0] != 0 || ptr[t][total] != nnz[t]) throw ArgError("r1cs: row pointers must run from 0 to nnz");
      for (uint64_t g = 0; g < total; g++)
        if (ptr[t][g + 1] < ptr[t][g]) throw ArgError("r1cs: row pointers must not decrease");
      for (uint64_t e = 0; e < nnz[t]; e++)
        if (cols[t][e] >= (1ull << logm)) throw ArgError("r1cs: a column is not below 2^logm");
      GBZ_CUDA(cudaMalloc(&m->ptr[t], 4 * (total + 1)));
      GBZ_CUDA(cudaMalloc(&m->cols[t], 4 * std::max<uint64_t>(nnz[t], 1)));
      GBZ_CUDA(cudaMemcpy(m->ptr[t], ptr[t], 4 * (total + 1), cudaMemcpyHostToDevice));
      if (nnz[t]) GBZ_CUDA(cudaMemcpy(m->cols[t], cols[t], 4 * nnz[t], cudaMemcpyHostToDevice));
      m->nnz[t] = nnz[t];
    }
  } catch (...) {
    for (int t = 0; t < 3; t++) {
      if (m->ptr[t]) cudaFree(m->ptr[t]);
      if (m->cols[t]) cudaFree(m->cols[t]);
    }
    throw;
  }
  *out = m.release();
  API_END(ctx)
}

gbz_status gbz_r1cs_free(gbz_r1cs *m) {
  if (!m) return GBZ_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(m->device);
  for (int t = 0; t < 3; t++) {
    if (m->ptr[t]) cudaFree(m->ptr[t]);
    if (m->cols[t]) cudaFree(m->cols[t]);
  }
  if (prev >= 0) cudaSetDevice(prev);
  delete m;
  return GBZ_OK;
}

gbz_status gbz_r1cs_reduce(gbz_ctx *ctx, const gbz_r1cs *m, const uint64_t *r, int nr, const int *degrees1,
                           int ndeg1, uint64_t *RA, uint64_t *RB, uint64_t *RC, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(m, "r1cs");
  need(r, "r");
  need(RA, "RA");
  need(RB, "RB");
  need(RC, "RC");
  check_degrees(degrees1, ndeg1, "r1cs reduce");
  if (nr != ndeg1) throw ArgError("r1cs reduce: r must have one entry per degree");
  const cudaStream_t s = ctx->stream;
  OpenBufs ob;
  const std::vector<fe> hr = read_fes(ctx, r, nr, mem);
  fe *beta1, *beta2;
  const int logS = reduce_tables(ctx, ob, m->N, m->logm, hr, degrees1, ndeg1, beta1, beta2, s);
  const uint64_t total = (uint64_t)m->N * m->rows;
  uint64_t *outs[3] = {RA, RB, RC};
  for (int t = 0; t < 3; t++) {
    R1csView v{};
    v.ptr[0] = m->ptr[t];
    v.cols[0] = m->cols[t];
    v.w[0] = fe_one();
    fe *o = mem == GBZ_MEM_DEVICE ? (fe *)outs[t] : ob.alloc<fe>(total);
    k_r1cs_rows<<<nblk(total), 256, 0, s>>>(v, total, beta1, beta2, logS, fe_one(), o);
    GBZ_CUDA(cudaGetLastError());
    if (mem == GBZ_MEM_HOST) GBZ_CUDA(cudaMemcpyAsync(outs[t], o, 16 * total, cudaMemcpyDeviceToHost, s));
  }
  GBZ_CUDA(cudaStreamSynchronize(s));
  API_END(ctx)
}

uint64_t gbz_piop_phase1_bytes(int N, uint64_t n, const int *degrees, int ndeg) {
  if (N < 4 || !is_pow2((uint64_t)N) || !is_pow2(n) || !degrees || ndeg < 1) return 0;
  return phase1_head_bytes(N, n) + cosumcheck_bytes(GBZ_SC_CUBIC, N, degrees, ndeg);
}

uint64_t gbz_piop_phase2_bytes(int N, const int *degrees2, int ndeg2) {
  if (N < 4 || !is_pow2((uint64_t)N) || !degrees2 || ndeg2 < 1) return 0;
  return 8 + 48 + cosumcheck_bytes(GBZ_SC_QUADRATIC, N, degrees2, ndeg2);
}

gbz_status gbz_piop_phase1(gbz_ctx *ctx, int N, uint64_t n, const uint64_t *vL, const uint64_t *vR,
                           const uint64_t *vO, const uint64_t *masks, const uint64_t *R1, const int *degrees,
                           int ndeg, uint64_t *fs, uint64_t *claims, uint64_t *ip, uint64_t *ip_b1,
                           uint64_t *vectors, uint32_t *flags, uint8_t *transcript, uint64_t capacity, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(vL, "vL");
  need(vR, "vR");
  need(vO, "vO");
  need(masks, "masks");
  need(R1, "R1");
  need(fs, "fs");
  need(claims, "claims");
  check_parties(N);
  check_degrees(degrees, ndeg, "piop phase 1");
  check_pow2(n, "piop phase 1: n");
  if (n < 4) throw ArgError("piop phase 1: n below the four mask entries");
  uint64_t prod = 1;
  Segs sg{};
  sg.n = ndeg;
  for (int i = 0; i < ndeg; i++) {
    prod *= (uint64_t)degrees[i];
    sg.off[i + 1] = sg.off[i] + 4u * (uint32_t)degrees[i];
  }
  if (prod != 2 * n) throw ArgError("piop phase 1: the degrees must multiply to 2 n");
  const uint64_t rlen = sg.off[ndeg];
  const uint64_t bytes = gbz_piop_phase1_bytes(N, n, degrees, ndeg);
  if (transcript && capacity < bytes) throw ArgError("piop phase 1: transcript capacity too small");
  const cudaStream_t s = ctx->stream;
  const int ln = ilog2(n), lk = ilog2((uint64_t)(N / 4)), k = N / 4;
  OpenBufs ob;
  {
    std::string key = "piop1:" + std::to_string(N) + ":" + std::to_string(n) + ":" + std::to_string(mem);
    for (int i = 0; i < ndeg; i++) key += ":" + std::to_string(degrees[i]);
    ob.pool = &ctx->pools[key];
  }
  // the draws: _r1 (log2 n), _r2 (log2 N/4), then r1's last entry
  fe hfs = read_fe(ctx, fs, mem);
  std::vector<fe> dr(ln + lk + 1);
  for (auto &x : dr) x = draw(hfs);
  std::vector<fe> r1(dr.begin(), dr.begin() + ln), r2(dr.begin() + ln, dr.begin() + ln + lk);
  r1.push_back(dr.back());
  // b2 = precompute_beta(_r2); the leader's weights of the parties' values
  std::vector<fe> b2(k);
  for (int i = 0; i < k; i++) {
    fe v = fe_one();
    for (int t = 0; t < lk; t++) v = fmul(v, ((i >> t) & 1) ? r2[t] : fsub(fe_one(), r2[t]));
    b2[i] = v;
  }
  const std::vector<fe> lambda = aggregate_weights(N, b2.data());
  // _beta(i, _r1) for the four mask positions (utils.cpp:1323-1335)
  fe bt[4];
  for (int i = 0; i < 4; i++) {
    fe v = fe_one();
    for (int t = 0; t < ln; t++) v = fmul(v, ((i >> t) & 1) ? r1[t] : fsub(fe_one(), r1[t]));
    bt[i] = v;
  }
  // transcript head: the draws, then the y record (filled on the device)
  HostRecs hr;
  const uint64_t off_d = hr.add(T_PIOP_DRAWS, (uint32_t)dr.size(), 16);
  for (size_t i = 0; i < dr.size(); i++) hr.put(off_d + 16 * i, dr[i]);
  const uint64_t off_y = hr.add(T_PIOP_Y, (uint32_t)(N + 2), 16);
  uint8_t *tr = ob.alloc<uint8_t>(bytes);
  GBZ_CUDA(cudaMemcpyAsync(tr, hr.bytes.data(), hr.bytes.size(), cudaMemcpyHostToDevice, s));
  // inputs on the device
  const fe *dvL = in_view(ctx, ob, (const fe *)vL, (uint64_t)N * n, mem);
  const fe *dvR = in_view(ctx, ob, (const fe *)vR, (uint64_t)N * n, mem);
  const fe *dvO = in_view(ctx, ob, (const fe *)vO, (uint64_t)N * n, mem);
  const fe *dm = in_view(ctx, ob, (const fe *)masks, 12ull * N, mem);
  const fe *dR1 = in_view(ctx, ob, (const fe *)R1, (uint64_t)N * rlen, mem);
  fe *dl = ob.alloc<fe>(N), *dy = ob.alloc<fe>(3);
  GBZ_CUDA(cudaMemcpyAsync(dl, lambda.data(), 16ull * N, cudaMemcpyHostToDevice, s));
  k_piop_y<<<1, kPiopMaxParties, 0, s>>>(dm, dR1, rlen, sg, N, bt[0], bt[1], bt[2], bt[3], dl, r1.back(), dy, tr,
                                         off_y);
  GBZ_CUDA(cudaGetLastError());
  fe hy[3];
  GBZ_CUDA(cudaMemcpyAsync(hy, dy, sizeof hy, cudaMemcpyDeviceToHost, s));
  // the masked, doubled vectors
  fe *P = ob.alloc<fe>(3ull * N * 2 * n);
  k_piop_extend<<<dim3(nblk(2 * n), N, 3), 256, 0, s>>>(dvL, dvR, dvO, dm, n, N, P);
  GBZ_CUDA(cudaGetLastError());
  GBZ_CUDA(cudaStreamSynchronize(s));
  // cubic_coSumcheck(vL, vR, vO, r1, r2, R1, y, K_r, degrees) (coPIOP.cpp:311-312)
  fe *ipb = ob.alloc<fe>(rlen);
  const uint64_t vn = (uint64_t)N * 2 * n;
  const CoscOut res = cosumcheck_run(ctx, GBZ_SC_CUBIC, N, 2 * n, P, P + vn, P + 2 * vn, dR1,
                                     cudaMemcpyDeviceToDevice, r1.data(), (int)r1.size(), r2.data(), hy[2], hy[1],
                                     degrees, ndeg, hfs, tr + hr.bytes.size(), cudaMemcpyDeviceToDevice, ipb);
  // sumcheck1_ip: ip_vec scaled by each party's share of the Lagrange vector
  // over N/4 points at the final challenge (coPIOP.cpp:314-328)
  const std::vector<fe> b1 = host_lagrange(res.claims[1], lk);
  const std::vector<fe> sc = share_scalars(b1, N);
  fe *dsc = ob.alloc<fe>(N), *dip = ob.alloc<fe>((uint64_t)N * rlen);
  GBZ_CUDA(cudaMemcpyAsync(dsc, sc.data(), 16ull * N, cudaMemcpyHostToDevice, s));
  k_scale_parties<<<dim3(nblk(rlen), N), 256, 0, s>>>(ipb, rlen, dsc, dip, rlen, 0);
  GBZ_CUDA(cudaGetLastError());
  put_out(ctx, claims, res.claims.data(), 16 * res.claims.size(), mem, false);
  put_out(ctx, fs, &res.fs, 16, mem, false);
  put_out(ctx, ip, dip, 16ull * N * rlen, mem, true);
  put_out(ctx, ip_b1, b1.data(), 16ull * k, mem, false);
  put_out(ctx, vectors, P, 16ull * 3 * vn, mem, true);
  put_out(ctx, transcript, tr, bytes, mem, true);
  GBZ_CUDA(cudaStreamSynchronize(s));
  if (flags) *flags = res.flags;
  API_END(ctx)
}

gbz_status gbz_piop_phase2(gbz_ctx *ctx, int N, uint64_t nw, const uint64_t *w, const uint64_t *masks,
                           const gbz_r1cs *m, int mask_l, const uint64_t *R2, const uint64_t *point1,
                           const uint64_t *evals1, const int *degrees1, int ndeg1, const int *degrees2, int ndeg2,
                           const uint64_t *K, uint64_t *fs, uint64_t *claims, uint64_t *abc, uint64_t *ip2,
                           uint64_t *ip3, uint64_t *ip_b1, uint64_t *vectors, uint32_t *flags, uint8_t *transcript,
                           uint64_t capacity, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(w, "w");
  need(masks, "masks");
  need(m, "r1cs");
  need(R2, "R2");
  need(point1, "point1");
  need(evals1, "evals1");
  need(K, "K");
  need(fs, "fs");
  need(claims, "claims");
  check_parties(N);
  if (m->N != N) throw ArgError("piop phase 2: the R1CS rows are split over another party count");
  check_degrees(degrees1, ndeg1, "piop phase 2: degrees1");
  check_degrees(degrees2, ndeg2, "piop phase 2: degrees2");
  check_pow2(nw, "piop phase 2: nw");
  if (degrees1[ndeg1 - 1] != 2) throw ArgError("piop phase 2: the first phase's last degree must be 2");
  const int k = N / 4, lk = ilog2((uint64_t)k);
  if (m->rows % k) throw ArgError("piop phase 2: rows per party must be a multiple of N/4");
  const uint64_t len = (uint64_t)N * m->rows / k;  // the reshared vector
  uint64_t nvl = 1;                                 // the beta shares: prod of degrees1 but the last
  for (int i = 0; i + 1 < ndeg1; i++) nvl *= (uint64_t)degrees1[i];
  const uint64_t seg = 2 * len / 32;
  if (2 * len % 32 || mask_l < 0 || seg <= (uint64_t)mask_l || 32 * (seg - mask_l) < len)
    throw ArgError("piop phase 2: the reshared vector does not fit 32 segments with mask_l gaps");
  if (2 * len + 4 * nvl != 2 * nw) throw ArgError("piop phase 2: |w| does not match the reduced and beta vectors");
  Segs sg2{};
  sg2.n = ndeg2;
  for (int i = 0; i < ndeg2; i++) sg2.off[i + 1] = sg2.off[i] + 2u * (uint32_t)degrees2[i];
  const uint64_t rlen = sg2.off[ndeg2];
  if (degrees2[0] < 4) throw ArgError("piop phase 2: degrees2[0] below the four mask entries");
  const uint64_t bytes = gbz_piop_phase2_bytes(N, degrees2, ndeg2);
  if (transcript && capacity < bytes) throw ArgError("piop phase 2: transcript capacity too small");
  const cudaStream_t s = ctx->stream;
  OpenBufs ob;
  {
    std::string key = "piop2:" + std::to_string(N) + ":" + std::to_string(nw) + ":" + std::to_string(mem) + ":" +
                      std::to_string(m->rows);
    for (int i = 0; i < ndeg1; i++) key += ":" + std::to_string(degrees1[i]);
    for (int i = 0; i < ndeg2; i++) key += "/" + std::to_string(degrees2[i]);
    ob.pool = &ctx->pools[key];
  }
  const std::vector<fe> r = read_fes(ctx, point1, ndeg1 + 1, mem);
  const std::vector<fe> y = read_fes(ctx, evals1, 3, mem);
  const fe hK = read_fe(ctx, K, mem);
  fe hfs = read_fe(ctx, fs, mem);
  const std::vector<fe> rr(r.begin(), r.end() - 1);  // _r: the point without its last entry
  // a, b, c (coPIOP.cpp:428-430)
  const fe a = draw(hfs), b = draw(hfs), c = draw(hfs);
  const std::vector<fe> Ll = host_lagrange(r.back(), 1);
  HostRecs hr;
  const uint64_t off_abc = hr.add(T_PIOP_ABC, 3, 16);
  hr.put(off_abc, a);
  hr.put(off_abc + 16, b);
  hr.put(off_abc + 32, c);
  uint8_t *tr = ob.alloc<uint8_t>(bytes);
  GBZ_CUDA(cudaMemcpyAsync(tr, hr.bytes.data(), hr.bytes.size(), cudaMemcpyHostToDevice, s));
  const fe *dw = in_view(ctx, ob, (const fe *)w, (uint64_t)N * nw, mem);
  const fe *dm = in_view(ctx, ob, (const fe *)masks, 12ull * N, mem);
  const fe *dR2 = in_view(ctx, ob, (const fe *)R2, (uint64_t)N * rlen, mem);
  // R_aggr = L_last[0] (a RA + b RB + c RC) (coPIOP.cpp:419-445)
  fe *beta1, *beta2;
  const int logS = reduce_tables(ctx, ob, N, m->logm, rr, degrees1, ndeg1, beta1, beta2, s);
  const uint64_t total = (uint64_t)N * m->rows;
  fe *aggr = ob.alloc<fe>(total);
  R1csView v{};
  for (int t = 0; t < 3; t++) {
    v.ptr[t] = m->ptr[t];
    v.cols[t] = m->cols[t];
  }
  v.w[0] = a;
  v.w[1] = b;
  v.w[2] = c;
  k_r1cs_rows<<<nblk(total), 256, 0, s>>>(v, total, beta1, beta2, logS, Ll[0], aggr);
  GBZ_CUDA(cudaGetLastError());
  // the second coSumcheck's vectors: P1 = (w, rL'), P2 = (segments of the
  // reshared R_aggr, beta shares L_last[1], zeros)
  fe *P = ob.alloc<fe>(2ull * N * 2 * nw);
  fe *P1 = P, *P2 = P + (uint64_t)N * 2 * nw;
  k_piop_p1<<<dim3(nblk(2 * nw), N), 256, 0, s>>>(dw, nw, dm, a, b, c, P1);
  GBZ_CUDA(cudaMemsetAsync(P2, 0, 16ull * N * 2 * nw, s));
  const std::vector<fe> mu = shamir_share_matrix(N);
  fe *dmu = ob.alloc<fe>(mu.size());
  GBZ_CUDA(cudaMemcpyAsync(dmu, mu.data(), 16 * mu.size(), cudaMemcpyHostToDevice, s));
  k_reshare_segments<<<dim3(nblk(len), N), 256, 0, s>>>(aggr, m->rows, N, dmu, seg, seg - mask_l, P2, 2 * nw);
  GBZ_CUDA(cudaGetLastError());
  // compute_beta_shares_multivariate (coPIOP.cpp:348-379) times L_last[1]
  std::vector<int> bd(degrees1, degrees1 + ndeg1 - 1);
  std::vector<fe> bp(rr.begin() + 1, rr.end());
  fe *bsh = ob.alloc<fe>(nvl), *t0 = ob.alloc<fe>(nvl), *t1 = ob.alloc<fe>(nvl);
  lagrange_tensor(ctx, bd, bp, bsh, t0, t1, s);
  std::vector<fe> bs = share_scalars(host_lagrange(rr[0], lk), N);
  for (auto &x : bs) x = fmul(x, Ll[1]);
  fe *dbs = ob.alloc<fe>(N);
  GBZ_CUDA(cudaMemcpyAsync(dbs, bs.data(), 16ull * N, cudaMemcpyHostToDevice, s));
  k_scale_parties<<<dim3(nblk(nvl), N), 256, 0, s>>>(bsh, nvl, dbs, P2, 2 * nw, 2 * len);
  GBZ_CUDA(cudaGetLastError());
  // quadratic_coSumcheck(w, R_aggr, R2, a yL + b yR + c yO, K_r, degrees2) (coPIOP.cpp:495-496)
  const fe K2 = fadd(fadd(fmul(a, y[0]), fmul(b, y[1])), fmul(c, y[2]));
  fe *ipb = ob.alloc<fe>(rlen);
  const CoscOut res = cosumcheck_run(ctx, GBZ_SC_QUADRATIC, N, 2 * nw, P1, P2, nullptr, dR2, cudaMemcpyDeviceToDevice,
                                     nullptr, 0, nullptr, K2, hK, degrees2, ndeg2, hfs, tr + hr.bytes.size(),
                                     cudaMemcpyDeviceToDevice, ipb);
  // sumcheck2_ip and sumcheck3_ip (coPIOP.cpp:562-604)
  const int cols = ndeg2 + 2;
  const std::vector<fe> b1 = host_lagrange(res.claims[1], lk);
  const std::vector<fe> sc = share_scalars(b1, N);
  fe *dsc = ob.alloc<fe>(N), *dip = ob.alloc<fe>((uint64_t)N * rlen);
  GBZ_CUDA(cudaMemcpyAsync(dsc, sc.data(), 16ull * N, cudaMemcpyHostToDevice, s));
  k_scale_parties<<<dim3(nblk(rlen), N), 256, 0, s>>>(ipb, rlen, dsc, dip, rlen, 0);
  GBZ_CUDA(cudaGetLastError());
  std::vector<fe> L = host_lagrange_head(res.claims[2], ilog2((uint64_t)degrees2[0]), 4);
  for (int i = 1; i < ndeg2; i++) {
    const fe t0v = host_lagrange0(res.claims[2 + i], ilog2((uint64_t)degrees2[i]));
    for (auto &x : L) x = fmul(x, t0v);
  }
  std::vector<fe> i3((size_t)N * 12);
  const fe wts[3] = {a, b, c};
  for (int p = 0; p < N; p++)
    for (int t = 0; t < 3; t++)
      for (int i = 0; i < 4; i++) i3[(size_t)p * 12 + 4 * t + i] = fmul(fmul(wts[t], L[i]), sc[p]);
  // claims[1].first = L_last[0]^{-1} claims[1].first (coPIOP.cpp:625)
  std::vector<fe> cl = res.claims;
  cl[cols] = fmul(finv(Ll[0]), cl[cols]);
  put_out(ctx, claims, cl.data(), 16 * cl.size(), mem, false);
  put_out(ctx, fs, &res.fs, 16, mem, false);
  const fe habc[3] = {a, b, c};
  put_out(ctx, abc, habc, 48, mem, false);
  put_out(ctx, ip2, dip, 16ull * N * rlen, mem, true);
  put_out(ctx, ip3, i3.data(), 16 * i3.size(), mem, false);
  put_out(ctx, ip_b1, b1.data(), 16ull * k, mem, false);
  put_out(ctx, vectors, P, 16ull * 2 * N * 2 * nw, mem, true);
  put_out(ctx, transcript, tr, bytes, mem, true);
  GBZ_CUDA(cudaStreamSynchronize(s));
  if (flags) *flags = res.flags;
  API_END(ctx)
}

}  // extern "C"
