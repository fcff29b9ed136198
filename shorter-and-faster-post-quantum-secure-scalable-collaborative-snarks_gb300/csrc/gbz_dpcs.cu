// The distributed PCS commitments of N parties on one device: Batch_dCommit
// and dCommit (distributed_PCS.cpp:56-170), whose codewords come from the
// reference's distributed FFT (distributed_batch_FFT / distributed_FFT,
// MPI_utils.cpp:2911-3298) and whose trees are built per party
// (distributed_commit, coPCS.cpp:311-367).
//
// The distributed FFT of N ranks is one transform of length N L over a
// message interleaved across the parties: party p's entry t is coefficient
// t N + p, and party r ends up holding, for every m < N, the block of L/N
// outputs starting at r L/N + m L.  Here each batch row is gathered into
// that interleaved order (one launch for all rows and parties), transformed
// once at length N L (one batched launch sequence for all rows) and
// scattered back into every party's layout; the column hashes and each
// party's tree follow.
#include <cmath>
#include <cstring>
#include <vector>

#include "gbz_copcs.cuh"
#include "gbz_ctx.cuh"

using namespace gbz_api;

namespace gbz {
namespace {

unsigned nblk2(uint64_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

// G_k[t N + p] = arr_p[k S + t] for t < S: row k of the interleaved message.
__global__ void k_dpcs_gather(const fe *arr, uint64_t A, uint64_t S, int N, fe *G) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;  // index in the row, t N + p
  if (i >= S * N) return;
  const int k = blockIdx.y;
  const uint64_t t = i / N, p = i % N;
  G[(uint64_t)k * S * N + i] = arr[p * A + (uint64_t)k * S + t];
}

// Party r's row k: out[r][k][m L/N + j] = X_k[r L/N + j + m L], j < L/N.
__global__ void k_dpcs_scatter(const fe *X, uint64_t L, int N, int rows, fe *out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;  // position in the party's row
  if (i >= L) return;
  const int k = blockIdx.y, r = blockIdx.z;
  const uint64_t blk = L / N, m = i / blk, j = i % blk;
  out[((uint64_t)r * rows + k) * L + i] = X[(uint64_t)k * N * L + r * blk + j + m * L];
}

// Column hashes of every party: column j of a party's nrows x len rows is
// MT_commit_Blake over its nrows entries (merkle_tree.cpp:201-221): the
// leaf of its first four entries, then log2(nrows / 4) self-hashes (an
// inner node hashes its left child twice, merkle_tree.cpp:267-299).
__global__ void k_dpcs_columns(const fe *rows, int nrows, uint64_t len, uint64_t pstride, int col_levels,
                               uint8_t *levels, uint64_t lstride) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= len) return;
  const fe *c = rows + blockIdx.y * pstride + j;
  uint32_t m[16], h[8];
  fe4_words(c[0], c[len], c[2 * len], c[3 * len], m);
  blake3_block64(m, h);
  for (int lv = 0; lv < col_levels; lv++) {
    for (int k = 0; k < 8; k++) m[k] = m[8 + k] = h[k];
    blake3_block64(m, h);
  }
  uint4 *o = reinterpret_cast<uint4 *>(levels + blockIdx.y * lstride + 32 * j);
  o[0] = make_uint4(h[0], h[1], h[2], h[3]);
  o[1] = make_uint4(h[4], h[5], h[6], h[7]);
  (void)nrows;
}

// Every party's tree over its column hashes, its root, and the leader's root.
void trees(gbz_ctx *ctx, uint8_t *levels, uint64_t leaves, int N, uint8_t *roots_h, uint8_t *leader_h) {
  const cudaStream_t s = ctx->stream;
  const uint64_t nh = 2 * leaves - 1;
  merkle_from_leaves_launch(levels, leaves, s, N);
  // every party's root (the last hash of its levels) in one strided copy
  std::vector<uint8_t> roots((size_t)32 * N);
  GBZ_CUDA(cudaMemcpy2DAsync(roots.data(), 32, levels + (nh - 1) * 32, 32 * nh, 32, N, cudaMemcpyDeviceToHost, s));
  GBZ_CUDA(cudaStreamSynchronize(s));
  if (roots_h) std::memcpy(roots_h, roots.data(), roots.size());
  // rank 0's tree over {its root, 0, ..., 0} (coPCS.cpp:338-349, distributed_PCS.cpp:101-110)
  if (leader_h) gbz_leader_root(roots.data(), N, leader_h);
}

void check_common(int N, uint64_t A, int rate) {
  if (N < 8 || N > 64 || !is_pow2((uint64_t)N)) throw ArgError("dpcs: N must be a power of two in [8, 64]");
  if (!is_pow2(A)) throw ArgError("dpcs: the parties' arrays must have a power-of-two length");
  if (rate < 1 || !is_pow2((uint64_t)rate)) throw ArgError("dpcs: rate must be a power of two");
}

// Host views of the outputs: device pointers as given, host ones staged.
template <typename T>
T *out_view(OpenBufs &ob, T *p, uint64_t count, int mem) {
  return mem == GBZ_MEM_DEVICE ? p : ob.alloc<T>(count);
}

// The codewords of `rows` batch rows of every party: gather, one transform
// of length N L per row, scatter into [party][row][L].
void dpcs_codewords(gbz_ctx *ctx, OpenBufs &ob, const fe *darr, uint64_t A, int N, int rows, int rate, fe *cw) {
  const cudaStream_t s = ctx->stream;
  const uint64_t S = A / rows, L = S * rate, len = L * N;
  const int lg = ilog2(len);
  if (lg > kMaxNttLogN) throw ArgError("dpcs: the distributed transform is longer than 2^26");
  fe *G = ob.alloc<fe>((uint64_t)rows * S * N), *X = ob.alloc<fe>((uint64_t)rows * len);
  fe *tmp = lg > 13 ? ob.alloc<fe>((uint64_t)rows * len) : nullptr;
  k_dpcs_gather<<<dim3(nblk2(S * N), rows), 256, 0, s>>>(darr, A, S, N, G);
  GBZ_CUDA(cudaGetLastError());
  ntt_launch_rows(ctx->tables(lg), G, S * N, S * N, X, len, rows, tmp, false, s);
  k_dpcs_scatter<<<dim3(nblk2(L), rows, N), 256, 0, s>>>(X, L, N, rows, cw);
  GBZ_CUDA(cudaGetLastError());
}

}  // namespace
}  // namespace gbz

using namespace gbz;

extern "C" {

gbz_status gbz_dpcs_batch_commit(gbz_ctx *ctx, int N, uint64_t A, const uint64_t *arr, const uint64_t *arr2, int rate,
                                 int batch, uint64_t *commit_data, uint64_t *codewords, uint8_t *levels, uint8_t *roots,
                                 uint8_t *leader_root, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(arr, "arr");
  need(arr2, "arr2");
  check_common(N, A, rate);
  if (batch < 4 || batch > 64 || !is_pow2((uint64_t)batch) || (uint64_t)batch > A)
    throw ArgError("dpcs: batch must be a power of two in [4, 64] dividing the arrays");
  const cudaStream_t s = ctx->stream;
  OpenBufs ob;
  ob.pool = &ctx->pools["dpcs_batch:" + std::to_string(N) + ":" + std::to_string(A) + ":" + std::to_string(rate) +
                        ":" + std::to_string(batch) + ":" + std::to_string(mem)];
  const uint64_t S = A / batch, L = S * rate, nh = 2 * L - 1;
  const fe *darr = (const fe *)arr;
  if (mem == GBZ_MEM_HOST) {
    fe *d = ob.alloc<fe>((uint64_t)N * A);
    GBZ_CUDA(cudaMemcpyAsync(d, arr, 16ull * N * A, cudaMemcpyHostToDevice, s));
    darr = d;
  } else {
    ob.alloc<uint8_t>(1);
  }
  fe *cw = out_view(ob, (fe *)codewords, (uint64_t)N * batch * L, mem);
  uint8_t *lv = out_view(ob, levels, 32ull * N * nh, mem);
  if (!cw) cw = ob.alloc<fe>((uint64_t)N * batch * L);
  if (!lv) lv = ob.alloc<uint8_t>(32ull * N * nh);
  dpcs_codewords(ctx, ob, darr, A, N, batch, rate, cw);
  // commit_data[i] = arr2's row i (distributed_PCS.cpp:63-69)
  if (commit_data) {
    const cudaMemcpyKind k = mem == GBZ_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToHost;
    GBZ_CUDA(cudaMemcpyAsync(commit_data, arr2, 16ull * N * A, k, s));
  }
  // column hashes over the batch rows (distributed_PCS.cpp:76-88), every party's tree
  k_dpcs_columns<<<dim3(nblk2(L), N), 256, 0, s>>>(cw, batch, L, (uint64_t)batch * L, ilog2((uint64_t)batch / 4), lv,
                                                   32 * nh);
  GBZ_CUDA(cudaGetLastError());
  trees(ctx, lv, L, N, roots, leader_root);
  if (mem == GBZ_MEM_HOST) {
    if (codewords) GBZ_CUDA(cudaMemcpyAsync(codewords, cw, 16ull * N * batch * L, cudaMemcpyDeviceToHost, s));
    if (levels) GBZ_CUDA(cudaMemcpyAsync(levels, lv, 32ull * N * nh, cudaMemcpyDeviceToHost, s));
  }
  GBZ_CUDA(cudaStreamSynchronize(s));
  API_END(ctx)
}

gbz_status gbz_dpcs_commit(gbz_ctx *ctx, int N, uint64_t A, const uint64_t *arr, int rate, uint64_t *codeword,
                           uint8_t *levels, uint8_t *roots, uint8_t *leader_root, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(arr, "arr");
  check_common(N, A, rate);
  const cudaStream_t s = ctx->stream;
  // the column height: plaintext_degrees[1] = 2^(log2 N - log2 N / 2) (distributed_PCS.cpp:42-43)
  const int lN = ilog2((uint64_t)N);
  const uint64_t d1 = 1ull << (lN - lN / 2);
  const uint64_t L = A * rate, leaves = L / d1, nh = 2 * leaves - 1;
  if (leaves < 1) throw ArgError("dpcs: codeword shorter than one column");
  OpenBufs ob;
  ob.pool = &ctx->pools["dpcs_single:" + std::to_string(N) + ":" + std::to_string(A) + ":" + std::to_string(rate) +
                        ":" + std::to_string(mem)];
  const fe *darr = (const fe *)arr;
  if (mem == GBZ_MEM_HOST) {
    fe *d = ob.alloc<fe>((uint64_t)N * A);
    GBZ_CUDA(cudaMemcpyAsync(d, arr, 16ull * N * A, cudaMemcpyHostToDevice, s));
    darr = d;
  } else {
    ob.alloc<uint8_t>(1);
  }
  fe *cw = out_view(ob, (fe *)codeword, (uint64_t)N * L, mem);
  uint8_t *lv = out_view(ob, levels, 32ull * N * nh, mem);
  if (!cw) cw = ob.alloc<fe>((uint64_t)N * L);
  if (!lv) lv = ob.alloc<uint8_t>(32ull * N * nh);
  dpcs_codewords(ctx, ob, darr, A, N, 1, rate, cw);
  // column i gathers codeword[j L/d1 + i], j < d1 (distributed_PCS.cpp:160-167)
  k_dpcs_columns<<<dim3(nblk2(leaves), N), 256, 0, s>>>(cw, (int)d1, leaves, L, ilog2(d1 / 4), lv, 32 * nh);
  GBZ_CUDA(cudaGetLastError());
  trees(ctx, lv, leaves, N, roots, leader_root);
  if (mem == GBZ_MEM_HOST) {
    if (codeword) GBZ_CUDA(cudaMemcpyAsync(codeword, cw, 16ull * N * L, cudaMemcpyDeviceToHost, s));
    if (levels) GBZ_CUDA(cudaMemcpyAsync(levels, lv, 32ull * N * nh, cudaMemcpyDeviceToHost, s));
  }
  GBZ_CUDA(cudaStreamSynchronize(s));
  API_END(ctx)
}

}  // extern "C"

// ---------------------------------------------------------------- opening

namespace gbz {
namespace {

enum : uint32_t {
  T_DPCS_EVAL_CLAIMS = 61, T_DPCS_DRAWS = 62, T_DPCS_ROOTS = 63, T_DPCS_QUERIES = 64, T_DPCS_POLY = 65,
  T_DPCS_CHALLENGE = 66, T_DPCS_K = 67, T_DPCS_WHIR_ROOT = 68
};

// out[p][k] = sum_h w[h] rows[p][h][k] (the row batching of commit data,
// distributed_PCS.cpp:1207-1213).
__global__ void k_rowsum(const fe *rows, int nrows, uint64_t len, const fe *w, fe *out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= len) return;
  const fe *r = rows + (uint64_t)blockIdx.y * nrows * len + k;
  fe acc = fe_zero();
  for (int h = 0; h < nrows; h++) acc = fadd(acc, fmul(w[h], r[(uint64_t)h * len]));
  out[(uint64_t)blockIdx.y * len + k] = acc;
}

// The row-batched global codeword from every party's codeword rows (party
// layout): X[r L/N + j + m L] = sum_h w[h] cw[r][h][m L/N + j]
// (distributed_PCS.cpp:1214-1219 on the reference's distributed layout).
__global__ void k_rowsum_global(const fe *cw, int nrows, uint64_t L, int N, const fe *w, fe *X) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;  // position in party r's row
  if (i >= L) return;
  const int r = blockIdx.y;
  const uint64_t blk = L / N, m = i / blk, j = i % blk;
  const fe *src = cw + (uint64_t)r * nrows * L + i;
  fe acc = fe_zero();
  for (int h = 0; h < nrows; h++) acc = fadd(acc, fmul(w[h], src[(uint64_t)h * L]));
  X[r * blk + j + m * L] = acc;
}

// One CTA per (i, j != i, party): sum_k b2_j[k] cdb_i[p][k] (the local
// part of the eval claims, :1223-1231).
__global__ void k_cross_dots(const fe *cdb, const fe *b2, uint64_t S, int P, int N, fe *out) {
  __shared__ fe red[256];
  const int p = blockIdx.x % N, pair = blockIdx.x / N;
  const int i = pair / (P - 1), jj = pair % (P - 1), j = jj < i ? jj : jj + 1;
  const fe *a = cdb + ((uint64_t)i * N + p) * S, *b = b2 + (uint64_t)j * S;
  fe acc = fe_zero();
  for (uint64_t k = threadIdx.x; k < S; k += blockDim.x) acc = fadd(acc, fmul(a[k], b[k]));
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fadd(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// arr[p] = sum_l w[l] cdb[l][p]; betas[p] = sum_l v[l][p] b2_l (v: the
// parties' weights b1_l[p] times a_l, :1290-1301).
__global__ void k_batch_vectors(const fe *cdb, const fe *b2, uint64_t S, int P, int N, fe w1, fe w2, const fe *v,
                                fe *arr, fe *betas) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S) return;
  const int p = blockIdx.y;
  const fe w[3] = {fe_one(), w1, w2};
  fe a = fe_zero(), bt = fe_zero();
  for (int l = 0; l < P; l++) {
    a = fadd(a, fmul(w[l], cdb[((uint64_t)l * N + p) * S + k]));
    bt = fadd(bt, fmul(v[l * N + p], b2[(uint64_t)l * S + k]));
  }
  arr[(uint64_t)p * S + k] = a;
  betas[(uint64_t)p * S + k] = bt;
}

// X = sum_l w[l] Xl[l] over n entries.
__global__ void k_combine3(const fe *Xl, uint64_t n, int P, fe w1, fe w2, fe *X) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const fe w[3] = {fe_one(), w1, w2};
  fe acc = fe_zero();
  for (int l = 0; l < P; l++) acc = fadd(acc, fmul(w[l], Xl[(uint64_t)l * n + i]));
  X[i] = acc;
}

// Party r's slice of the global codeword in the distributed layout: for
// m < nb, the L/N entries from r L/N + m L.
__global__ void k_party_slices(const fe *X, uint64_t L, int N, uint64_t len, fe *out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  const int r = blockIdx.y;
  const uint64_t blk = L / N, m = i / blk, j = i % blk;
  out[(uint64_t)r * len + i] = X[r * blk + j + m * L];
}

std::vector<fe> host_lag(fe r, int logd) {
  const uint64_t d = 1ull << logd;
  std::vector<fe> pw(d), out(d);
  pw[0] = fe_one();
  for (uint64_t j = 1; j < d; j++) pw[j] = fmul(pw[j - 1], r);
  const fe wi = finv(root_of_unity(logd)), dinv = finv(fe_make(d, 0));
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

std::vector<fe> host_beta(const fe *r, int nr) {
  std::vector<fe> b(1ull << nr);
  for (uint64_t x = 0; x < b.size(); x++) {
    fe v = fe_one();
    for (int t = 0; t < nr; t++) v = fmul(v, ((x >> t) & 1) ? r[t] : fsub(fe_one(), r[t]));
    b[x] = v;
  }
  return b;
}

struct Recs {
  std::vector<uint8_t> b;
  void add(uint32_t tag, uint32_t count, const void *payload, uint64_t bytes) {
    const uint64_t at = b.size();
    b.resize(at + 8 + bytes);
    std::memcpy(&b[at], &tag, 4);
    std::memcpy(&b[at + 4], &count, 4);
    if (bytes) std::memcpy(&b[at + 8], payload, bytes);
  }
};

std::vector<int> fold_degrees(int N) {
  const int lN = ilog2((uint64_t)N);
  std::vector<int> d(1, 1 << (lN - lN / 2));
  if ((1 << (lN / 2)) > 1) d.push_back(1 << (lN / 2));
  return d;
}

int plain_queries(int rate) { return (int)(-100.0 / log2(sqrt(1.0 / (double)rate))); }

// A device array to the caller (device memory, or host memory by mem).
void put_dev(gbz_ctx *ctx, void *dst, const void *src, uint64_t bytes, int mem) {
  if (!dst || !bytes) return;
  GBZ_CUDA(cudaMemcpyAsync(dst, src, bytes, mem == GBZ_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                           ctx->stream));
}

// One commitment of the opening: every party's slice of the global codeword
// X (length N L / D), its columns of d entries spaced |slice| / d, every
// party's tree; the leader's root (over N zero leaves, coPCS.cpp:398-408);
// then get_indexes' draws over M positions (Fiat_Shamir.cpp:37-53).
void commit_round(gbz_ctx *ctx, OpenBufs &ob, const fe *X, uint64_t L, int N, uint64_t D, int d, int l, uint64_t M,
                  fe &fs, Recs &rec) {
  const cudaStream_t s = ctx->stream;
  const uint64_t len = L / D, leaves = len / d, nh = 2 * leaves - 1;
  fe *sl = ob.alloc<fe>((uint64_t)N * len);
  uint8_t *lv = ob.alloc<uint8_t>(32ull * N * nh);
  k_party_slices<<<dim3(nblk2(len), N), 256, 0, s>>>(X, L, N, len, sl);
  k_dpcs_columns<<<dim3(nblk2(leaves), N), 256, 0, s>>>(sl, d, leaves, len, ilog2((uint64_t)d / 4), lv, 32 * nh);
  GBZ_CUDA(cudaGetLastError());
  std::vector<uint8_t> roots(32ull * (N + 1));
  trees(ctx, lv, leaves, N, roots.data(), nullptr);
  uint8_t zero[32] = {0};
  gbz_leader_root(zero, N, roots.data() + 32ull * N);
  rec.add(T_DPCS_ROOTS, (uint32_t)(N + 1), roots.data(), roots.size());
  std::vector<uint32_t> q(2 * (size_t)l);
  for (int i = 0; i < l; i++) {
    fs = hash_F(fs, fs);
    q[2 * i] = (uint32_t)(fs.re % (uint64_t)N);
    q[2 * i + 1] = (uint32_t)(fs.im % M);
  }
  rec.add(T_DPCS_QUERIES, (uint32_t)(2 * l), q.data(), 4 * q.size());
}

}  // namespace
}  // namespace gbz

extern "C" {

uint64_t gbz_dpcs_open_bytes(int N, int P, int rate) {
  if (N < 8 || N > 64 || !is_pow2((uint64_t)N) || (P != 2 && P != 3) || rate < 1) return 0;
  const std::vector<int> degs = gbz::fold_degrees(N);
  const int l = gbz::plain_queries(rate);
  uint64_t b = 8 + 16ull * P * (P - 1) + 8 + 64;
  for (size_t i = 0; i < degs.size(); i++) {
    b += (8 + 32ull * (N + 1)) + (8 + 8ull * l);                  // a commitment (the batched one, then FRI)
    b += (8 + 32ull * degs[i]) + (8 + 16) + (8 + 16);            // poly, challenge, K
  }
  return b + 8 + 32;
}

gbz_status gbz_dpcs_open(gbz_ctx *ctx, int N, int P, int rows, uint64_t S, int rate, const uint64_t *commit_data,
                         const uint64_t *codewords, const uint64_t *points, const uint64_t *claims, int verify,
                         int whir_rate, uint64_t *fs, uint64_t *arr_out, uint64_t *betas_out, uint64_t *K_out,
                         uint64_t *whir_codeword, uint8_t *whir_root, uint32_t *flags, uint8_t *transcript,
                         uint64_t capacity, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(commit_data, "commit_data");
  need(codewords, "codewords");
  need(points, "points");
  need(claims, "claims");
  need(fs, "fs");
  check_common(N, S, rate);
  if (P != 2 && P != 3) throw ArgError("dpcs open: 2 or 3 polynomials");
  if (rows < 1 || rows > 64 || !is_pow2((uint64_t)rows)) throw ArgError("dpcs open: rows must be a power of two <= 64");
  if (whir_rate < 2 || !is_pow2((uint64_t)whir_rate)) throw ArgError("dpcs open: WHIR rate must be a power of two");
  const std::vector<int> degs = fold_degrees(N);
  uint64_t Dall = 1;
  for (int d : degs) Dall *= (uint64_t)d;
  const uint64_t L = S * rate;
  if (S % Dall || L % ((uint64_t)N * Dall)) throw ArgError("dpcs open: data too short to fold");
  const uint64_t bytes = gbz_dpcs_open_bytes(N, P, rate);
  if (transcript && capacity < bytes) throw ArgError("dpcs open: transcript capacity too small");
  const cudaStream_t s = ctx->stream;
  const int lS = ilog2(S), lR = ilog2((uint64_t)rows), lN = ilog2((uint64_t)N), np = lS + lR + lN;
  const int l = plain_queries(rate);
  OpenBufs ob;
  ob.pool = &ctx->pools["dpcs_open:" + std::to_string(N) + ":" + std::to_string(P) + ":" + std::to_string(rows) + ":" +
                        std::to_string(S) + ":" + std::to_string(rate) + ":" + std::to_string(mem)];
  // inputs
  const uint64_t ncd = (uint64_t)P * N * rows * S, ncw = (uint64_t)P * N * rows * L;
  const fe *dcd = (const fe *)commit_data, *dcw = (const fe *)codewords;
  std::vector<fe> pts((size_t)P * np), ys(P);
  fe hfs;
  if (mem == GBZ_MEM_HOST) {
    fe *a = ob.alloc<fe>(ncd), *b = ob.alloc<fe>(ncw);
    GBZ_CUDA(cudaMemcpyAsync(a, commit_data, 16 * ncd, cudaMemcpyHostToDevice, s));
    GBZ_CUDA(cudaMemcpyAsync(b, codewords, 16 * ncw, cudaMemcpyHostToDevice, s));
    dcd = a;
    dcw = b;
    std::memcpy(pts.data(), points, 16 * pts.size());
    std::memcpy(ys.data(), claims, 16 * ys.size());
    hfs = fe_make(fs[0], fs[1]);
  } else {
    ob.alloc<uint8_t>(1);
    ob.alloc<uint8_t>(1);
    GBZ_CUDA(cudaMemcpyAsync(pts.data(), points, 16 * pts.size(), cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaMemcpyAsync(ys.data(), claims, 16 * ys.size(), cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaMemcpyAsync(&hfs, fs, 16, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaStreamSynchronize(s));
  }
  // each point as (r2: log2 S, r3: log2 rows, r1: log2 N) (:1188-1203);
  // the long beta (r2) on the device, the row and party betas on the host
  std::vector<fe> b3h((size_t)P * rows), b1h((size_t)P * N);
  for (int q = 0; q < P; q++) {
    const fe *r = pts.data() + (size_t)q * np;
    std::vector<fe> t3 = host_beta(r + lS, lR), t1 = host_beta(r + lS + lR, lN);
    std::copy(t3.begin(), t3.end(), b3h.begin() + (size_t)q * rows);
    std::copy(t1.begin(), t1.end(), b1h.begin() + (size_t)q * N);
  }
  fe *db2 = ob.alloc<fe>((uint64_t)P * S), *db3 = ob.alloc<fe>((uint64_t)P * rows), *dpts = ob.alloc<fe>(pts.size());
  GBZ_CUDA(cudaMemcpyAsync(dpts, pts.data(), 16 * pts.size(), cudaMemcpyHostToDevice, s));
  for (int q = 0; q < P; q++) beta_launch(dpts + (size_t)q * np, lS, db2 + (uint64_t)q * S, s);
  GBZ_CUDA(cudaMemcpyAsync(db3, b3h.data(), 16ull * P * rows, cudaMemcpyHostToDevice, s));
  // row batching of the data and of the codewords (global order)
  fe *cdb = ob.alloc<fe>((uint64_t)P * N * S), *cwb = ob.alloc<fe>((uint64_t)P * N * L);
  for (int q = 0; q < P; q++) {
    k_rowsum<<<dim3(nblk2(S), N), 256, 0, s>>>(dcd + (uint64_t)q * N * rows * S, rows, S, db3 + (uint64_t)q * rows,
                                              cdb + (uint64_t)q * N * S);
    k_rowsum_global<<<dim3(nblk2(L), N), 256, 0, s>>>(dcw + (uint64_t)q * N * rows * L, rows, L, N,
                                                     db3 + (uint64_t)q * rows, cwb + (uint64_t)q * N * L);
  }
  GBZ_CUDA(cudaGetLastError());
  // the eval claims: every party's cross evaluations, summed with b1_j[p]
  fe *dx = ob.alloc<fe>((uint64_t)P * (P - 1) * N);
  k_cross_dots<<<P * (P - 1) * N, 256, 0, s>>>(cdb, db2, S, P, N, dx);
  GBZ_CUDA(cudaGetLastError());
  std::vector<fe> hx((size_t)P * (P - 1) * N);
  GBZ_CUDA(cudaMemcpyAsync(hx.data(), dx, 16 * hx.size(), cudaMemcpyDeviceToHost, s));
  GBZ_CUDA(cudaStreamSynchronize(s));
  std::vector<fe> K((size_t)P * (P - 1), fe_zero());
  for (int i = 0; i < P; i++)
    for (int jj = 0; jj < P - 1; jj++) {
      const int j = jj < i ? jj : jj + 1;
      for (int p = 0; p < N; p++)
        K[(size_t)i * (P - 1) + jj] =
            fadd(K[(size_t)i * (P - 1) + jj], fmul(hx[((size_t)i * (P - 1) + jj) * N + p], b1h[(size_t)j * N + p]));
    }
  Recs rec;
  rec.add(T_DPCS_EVAL_CLAIMS, (uint32_t)K.size(), K.data(), 16 * K.size());
  // a = (hash_to_field(K), hash_to_field({0})), b = two draws, b[0] = 0 (:1259-1263)
  fe a0 = hfs;
  for (const fe &k : K) a0 = hash_F(a0, k);
  const fe a1 = hash_F(a0, fe_zero()), b0 = hash_F(a1, fe_zero()), b1 = hash_F(b0, fe_zero());
  hfs = b1;
  {
    const fe dr[4] = {a0, a1, b0, b1};
    rec.add(T_DPCS_DRAWS, 4, dr, sizeof dr);
  }
  fe y0;
  if (P == 3)
    y0 = fadd(fadd(fadd(ys[0], fmul(a0, K[0])), fmul(a1, K[1])),
              fmul(b1, fadd(fadd(K[4], fmul(a0, K[5])), fmul(a1, ys[2]))));
  else
    y0 = fadd(ys[0], fmul(a0, K[0]));
  // the batched data, the betas (weights a, times b1_l[p]) and the batched
  // codeword (weights {1, b[0] = 0, b[1]} as the reference passes them, :1291)
  std::vector<fe> vw((size_t)P * N);
  const fe aw[3] = {fe_one(), a0, a1};
  for (int q = 0; q < P; q++)
    for (int p = 0; p < N; p++) vw[(size_t)q * N + p] = fmul(aw[q], b1h[(size_t)q * N + p]);
  fe *dvw = ob.alloc<fe>((uint64_t)P * N), *arr = ob.alloc<fe>((uint64_t)N * S), *bet = ob.alloc<fe>((uint64_t)N * S);
  fe *tmpv = ob.alloc<fe>((uint64_t)N * S), *X = ob.alloc<fe>((uint64_t)N * L), *Xt = ob.alloc<fe>((uint64_t)N * L);
  GBZ_CUDA(cudaMemcpyAsync(dvw, vw.data(), 16 * vw.size(), cudaMemcpyHostToDevice, s));
  k_batch_vectors<<<dim3(nblk2(S), N), 256, 0, s>>>(cdb, db2, S, P, N, fe_zero(), b1, dvw, arr, bet);
  k_combine3<<<nblk2((uint64_t)N * L), 256, 0, s>>>(cwb, (uint64_t)N * L, P, fe_zero(), b1, X);
  GBZ_CUDA(cudaGetLastError());
  commit_round(ctx, ob, X, L, N, 1, degs[0], l, L, hfs, rec);
  // the rounds (:1365-1421)
  uint32_t fl = 0;
  fe Kc = y0;
  uint64_t n = S, D = 1;
  fe *H = ob.alloc<fe>((uint64_t)N * 64), *poly = ob.alloc<fe>(64), *dL = ob.alloc<fe>(32);
  fe *ones = ob.alloc<fe>(N);
  {
    std::vector<fe> o(N, fe_one());
    GBZ_CUDA(cudaMemcpyAsync(ones, o.data(), 16ull * N, cudaMemcpyHostToDevice, s));
  }
  bool stopped = false;
  for (size_t i = 0; i < degs.size(); i++) {
    const int d = degs[i], logd = ilog2((uint64_t)d), Dd = 2 * d;
    const uint64_t blocks = (uint64_t)N * n / d, pblocks = n / d;
    const NttTables &td = ctx->tables(logd), &tD = ctx->tables(logd + 1);
    fe *e1 = ob.alloc<fe>(blocks * Dd), *e2 = ob.alloc<fe>(blocks * Dd);
    ntt_batched(td, arr, d, (uint32_t)d, tmpv, blocks, true, s);
    ntt_batched(tD, tmpv, d, (uint32_t)d, e1, blocks, false, s);
    ntt_batched(td, bet, d, (uint32_t)d, tmpv, blocks, true, s);
    ntt_batched(tD, tmpv, d, (uint32_t)d, e2, blocks, false, s);
    const int lanes = Dd >= 256 ? 1 : 256 / Dd;
    const int per_cta = (int)std::max<uint64_t>((uint64_t)lanes, (pblocks + 607) / 608);
    fe *cpart = ob.alloc<fe>((uint64_t)N * Dd * cophase1_parts(pblocks, per_cta));
    cophase1_reduce_launch(e1, e2, nullptr, nullptr, nullptr, pblocks, logd + 1, per_cta, cpart, H, s, N);
    aggregate_launch(H, N, Dd, ones, poly, s);  // aggregate_plaintext_poly_batch: the plain sum
    std::vector<fe> hp(Dd);
    GBZ_CUDA(cudaMemcpyAsync(hp.data(), poly, 16ull * Dd, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaStreamSynchronize(s));
    fe ev = fe_zero();
    for (int j = 0; j < d; j++) ev = fadd(ev, hp[2 * j]);
    if (!fe_eq(ev, Kc) && verify) {
      fl |= 1;  // "Sumcheck Error Round": the reference returns here
      stopped = true;
      break;
    }
    for (const fe &x : hp) hfs = hash_F(hfs, x);
    const fe c = hfs;
    const std::vector<fe> L2 = host_lag(c, logd + 1), Ld = host_lag(c, logd);
    Kc = fe_zero();
    for (int j = 0; j < Dd; j++) Kc = fadd(Kc, fmul(hp[j], L2[j]));
    rec.add(T_DPCS_POLY, (uint32_t)Dd, hp.data(), 16ull * Dd);
    rec.add(T_DPCS_CHALLENGE, 1, &c, 16);
    rec.add(T_DPCS_K, 1, &Kc, 16);
    GBZ_CUDA(cudaMemcpyAsync(dL, Ld.data(), 16ull * d, cudaMemcpyHostToDevice, s));
    cophase2_launch(arr, (uint64_t)N * n, dL, logd, tmpv, s);
    GBZ_CUDA(cudaMemcpyAsync(arr, tmpv, 16ull * N * n / d, cudaMemcpyDeviceToDevice, s));
    cophase2_launch(bet, (uint64_t)N * n, dL, logd, tmpv, s);
    GBZ_CUDA(cudaMemcpyAsync(bet, tmpv, 16ull * N * n / d, cudaMemcpyDeviceToDevice, s));
    // RS_distributed_fold (coPCS_utils.cpp:440-504) is the multifold of the global codeword
    const uint64_t glen = (uint64_t)N * L / D;
    multifold5_launch(X, glen, dL, logd, Xt, ctx->tables(ilog2(glen)), s);
    std::swap(X, Xt);
    n /= d;
    D *= d;
    if (i + 1 < degs.size()) commit_round(ctx, ob, X, L, N, D, d, l, L / D / d, hfs, rec);
  }
  const uint64_t na = (uint64_t)N * n;
  if (!stopped) {
    // the leader: the gathered data (party by party), betas and codeword,
    // and Whir_Commit_initial of the data at the WHIR rate (Whir.cpp:158-190)
    fe *wc = ob.alloc<fe>(na * whir_rate);
    uint8_t *wl = ob.alloc<uint8_t>(32 * (na * whir_rate / 2 - 1));
    const gbz_status st = gbz_whir_commit(ctx, (const uint64_t *)arr, na, whir_rate, (uint64_t *)wc, wl,
                                          GBZ_MEM_DEVICE);
    if (st != GBZ_OK) throw ArgError("dpcs open: the leader's WHIR commitment failed");
    uint8_t root[32];
    GBZ_CUDA(cudaMemcpyAsync(root, wl + 32 * (na * whir_rate / 2 - 2), 32, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaStreamSynchronize(s));
    rec.add(T_DPCS_WHIR_ROOT, 1, root, 32);
    if (whir_root) std::memcpy(whir_root, root, 32);
    put_dev(ctx, arr_out, arr, 16 * na, mem);
    put_dev(ctx, betas_out, bet, 16 * na, mem);
    put_dev(ctx, whir_codeword, wc, 16 * na * whir_rate, mem);
    if (K_out) {
      if (mem == GBZ_MEM_DEVICE)
        GBZ_CUDA(cudaMemcpyAsync(K_out, &Kc, 16, cudaMemcpyHostToDevice, s));
      else
        std::memcpy(K_out, &Kc, 16);
    }
  }
  if (mem == GBZ_MEM_DEVICE)
    GBZ_CUDA(cudaMemcpyAsync(fs, &hfs, 16, cudaMemcpyHostToDevice, s));
  else
    std::memcpy(fs, &hfs, 16);
  if (transcript) {
    const cudaMemcpyKind k = mem == GBZ_MEM_DEVICE ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
    GBZ_CUDA(cudaMemcpyAsync(transcript, rec.b.data(), rec.b.size(), k, s));
  }
  GBZ_CUDA(cudaStreamSynchronize(s));
  if (flags) *flags = fl;
  API_END(ctx)
}

}  // extern "C"
