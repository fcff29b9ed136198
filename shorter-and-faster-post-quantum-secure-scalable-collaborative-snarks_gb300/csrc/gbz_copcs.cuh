// Launchers of the coPCS-side kernels (gbz_copcs.cu).
#pragma once
#include <vector>

#include "gbz_internal.cuh"

struct gbz_ctx;

namespace gbz {

// RS_multifold5 (coPCS_utils.cpp:386-437): out (n / 2^logd) from cw (n),
// fold weights a (2^logd, device); tn: twiddle tables of length n.
void multifold5_launch(const fe *cw, uint64_t n, const fe *a, int logd, fe *out, const NttTables &tn,
                       cudaStream_t s);
// out[i] = r^i for i < n.
void powers_launch(fe r, uint64_t n, fe *out, cudaStream_t s);
// x[j] *= omega_T^{-j} for j < n, T = 2^t.logn.
// rows vectors of n entries, row_stride apart
void coset_launch(fe *x, uint64_t n, const NttTables &t, cudaStream_t s, int rows = 1, uint64_t row_stride = 0);
// out[r L + rate t + off] = x[r n + t] for t < n, r < rows.
void strided_copy_launch(const fe *x, uint64_t n, fe *out, uint64_t L, int rate, int off, int rows, cudaStream_t s);
// distributed_MT (coPCS.cpp:152-202) of `parties` parties in the same
// launches: party p's rows at rows + p rows_stride, its levels (2L - 1
// hashes, column roots first) at levels + p (2L - 1) hashes and its leader
// root over 2^logN parties at root + 32 p.
void column_merkle_launch(const fe *rows, int nrows, uint64_t L, uint8_t *levels, int logN, uint8_t *root,
                          cudaStream_t s, int parties = 1, uint64_t rows_stride = 0);
// Packed Shamir shares (compute_secret_shares, MPI_utils.cpp:2738-2764).
std::vector<fe> shamir_share_matrix(int N);
void shares_launch(const fe *v, const fe *fill, uint64_t groups, int N, const fe *mu, fe *shares, cudaStream_t s);
// Leader aggregation of party messages (sumcheck_aggr, MPI_utils.cpp:2604-2670).
std::vector<fe> aggregate_weights(int N, const fe *b);
// The weights of g^T E for any g over the unpacked shares E.
std::vector<fe> aggregate_weights_even(int N, const std::vector<fe> &g);
void aggregate_launch(const fe *msgs, int N, uint64_t len, const fe *lambda, fe *out, cudaStream_t s);
// The same weights as aggregate_weights, computed on the device from b
// (N/4 weights, device) into lambda (N, device).
void aggregate_weights_launch(const fe *b, int N, fe *lambda, cudaStream_t s);
// coSumcheck phase 1 helpers; extended blocks of up to 2^13 entries (one
// batched transform per block).
constexpr int kMaxCoLogD = 13;
void nonzero_blocks_launch(const fe *v, uint64_t nblocks, int logd, uint8_t *flags, cudaStream_t s);
uint64_t cophase1_parts(uint64_t nblocks, int blocks_per_cta);
// parties > 1: that many parties one after the other in every array (e*:
// nblocks << logD entries each, flags: nblocks, partial:
// cophase1_parts(nblocks, blocks_per_cta) << logD, H: 1 << logD).
void cophase1_reduce_launch(const fe *e1, const fe *e2, const fe *e3, const fe *e4, const uint8_t *flags,
                            uint64_t nblocks, int logD, int blocks_per_cta, fe *partial, fe *H, cudaStream_t s,
                            int parties = 1);
// coSumcheck phase 2 (coSumcheck.cpp:66-148, 201-213).
void cophase2_launch(const fe *v, uint64_t n, const fe *L, int logd, fe *out, cudaStream_t s);

// quadratic_coSumcheck / cubic_coSumcheck of N parties (coSumcheck.cpp:
// 233-331, 335-448), the body of gbz_cosumcheck.  p1, p2, p3 (cubic), R:
// party-major arrays copied in with kin (the call folds copies); r1 (cubic,
// nr1 = log2 n entries), r2 (log2(N/4) entries), K, K_r, fs: host values.
// The transcript (cosumcheck_bytes) goes to `transcript` (may be null) by
// tr_kind; when ip is not null it receives the coSumcheck's inner-product
// vector ip_vec flattened (sum of (2 or 4) d_i entries, device).  Returns
// rows x (ndeg + 2) claim words [eval, r_final, r_0 .. r_{ndeg-1}] (rows = 5
// quadratic, 4 cubic), the chain state and the check flags.
struct CoscOut {
  std::vector<fe> claims;
  fe fs;
  uint32_t flags;
};
CoscOut cosumcheck_run(gbz_ctx *ctx, int form, int N, uint64_t n, const fe *p1, const fe *p2, const fe *p3,
                       const fe *R, cudaMemcpyKind kin, const fe *r1, int nr1, const fe *r2, fe K, fe K_r,
                       const int *degrees, int ndeg, fe fs, uint8_t *transcript, cudaMemcpyKind tr_kind, fe *ip);
uint64_t cosumcheck_bytes(int form, int N, const int *degrees, int ndeg);

}  // namespace gbz
