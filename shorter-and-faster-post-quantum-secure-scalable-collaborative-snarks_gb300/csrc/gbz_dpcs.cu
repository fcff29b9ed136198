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
  for (int p = 0; p < N; p++) merkle_from_leaves_launch(levels + (uint64_t)p * 32 * nh, leaves, s);
  std::vector<uint8_t> roots((size_t)32 * N);
  for (int p = 0; p < N; p++)
    GBZ_CUDA(cudaMemcpyAsync(roots.data() + 32 * p, levels + ((uint64_t)p * nh + nh - 1) * 32, 32,
                             cudaMemcpyDeviceToHost, s));
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
