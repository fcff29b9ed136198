// Kernels of the collaborative-PCS side of the prover: RS folding, the
// coPCS encoding, per-column Merkle hashing, packed Shamir shares, the
// leader's aggregation of party round messages, and the block-univariate
// (coSumcheck) rounds.
#include <vector>

#include "gbz_copcs.cuh"

namespace gbz {

namespace {

__device__ __forceinline__ fe pow_tab(const fe *lo, const fe *hi, uint64_t e) { return fmul(lo[e & 4095u], hi[e >> 12]); }

// RS_multifold5 (coPCS_utils.cpp:386-437): output i combines the d = 2^logd
// entries cw[i + t n/d] through log2(d) butterfly levels whose twiddles are
// powers of omega_n^{-1} (level 0: omega_n^{-j}; level lv: omega_n^{-2^lv j}
// for the kept index j), then y_i = d^{-1} sum_k a_k partial_i[k].
constexpr int kMaxFoldLog = 4;
// omega_n^{-(g step 2^lv) mod n} for level lv and group g (15 values for
// d = 16), so that every twiddle of an output is (omega_n^{-i})^{2^lv}
// times a constant: one table lookup per output instead of one per pair.
struct FoldConsts {
  fe c[kMaxFoldLog][1 << (kMaxFoldLog - 1)];
};
template <int LOGD>
__global__ void __launch_bounds__(256)
multifold5_kernel(const fe *cw, uint64_t n, const fe *a, fe *out, const fe *inv_lo, const fe *inv_hi, fe len_inv,
                  FoldConsts k) {
  constexpr int D = 1 << LOGD;
  const uint64_t nout = n >> LOGD;
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nout) return;
  const uint64_t half = n / 2, step = nout;
  fe buf[D], nb[D];
  fe wl = pow_tab(inv_lo, inv_hi, i);  // (omega^{-i})^{2^lv}
#pragma unroll
  for (int t = 0; t < D / 2; t++) {
    const uint64_t j = i + t * step;
    const fe x = cw[j], y = cw[j + half];
    buf[2 * t] = fadd(x, y);
    buf[2 * t + 1] = fmul(fmul(wl, k.c[0][t]), fsub(x, y));
  }
#pragma unroll
  for (int lv = 1; lv < LOGD; lv++) {
    wl = fmul(wl, wl);
    const int groups = D >> lv, ng = groups / 2, width = 1 << lv;
#pragma unroll
    for (int g = 0; g < ng; g++) {
      const fe po = fmul(wl, k.c[lv][g]);
#pragma unroll
      for (int q = 0; q < width; q++) {
        const fe x = buf[g * width + q], y = buf[(g + ng) * width + q];
        nb[g * 2 * width + q] = fadd(x, y);
        nb[g * 2 * width + q + width] = fmul(po, fsub(x, y));
      }
    }
#pragma unroll
    for (int q = 0; q < D; q++) buf[q] = nb[q];
  }
  fe acc = fe_zero();
#pragma unroll
  for (int q = 0; q < D; q++) acc = fadd(acc, fmul(a[q], buf[q]));
  out[i] = fmul(acc, len_inv);
}

__global__ void powers_kernel(fe r, uint64_t n, fe *out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = fpow(r, i);
}

// x[j] *= omega^{-j} for j < n (omega^{-e} from the inverse tables).
__global__ void coset_kernel(fe *x, uint64_t n, const fe *inv_lo, const fe *inv_hi, uint64_t row_stride) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  x += blockIdx.y * row_stride;
  if (j < n) x[j] = fmul(x[j], pow_tab(inv_lo, inv_hi, j));
}

// Column roots of distributed_MT (coPCS.cpp:168-176): the root of
// MT_commit_Blake over the 32-entry column depends only on its first leaf
// (rows 0..3), because every inner node hashes its left child twice; the
// other seven leaves the reference hashes are discarded, so they are not
// computed here.
__global__ void column_root_kernel(const fe *rows, int nrows, uint64_t L, uint8_t *roots, uint64_t rows_stride,
                                   uint64_t roots_stride) {
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= L) return;
  rows += rows_stride * blockIdx.y;  // grid.y: parties
  roots += roots_stride * blockIdx.y;
  fe e[4];
  for (int k = 0; k < 4; k++) e[k] = k < nrows ? rows[(uint64_t)k * L + j] : fe_zero();
  uint32_t m[16], h[8];
  fe4_words(e[0], e[1], e[2], e[3], m);
  blake3_block64(m, h);
  for (int lv = 0; lv < 3; lv++) {  // 8 leaves -> 4 -> 2 -> 1
    for (int k = 0; k < 8; k++) { m[k] = h[k]; m[8 + k] = h[k]; }
    blake3_block64(m, h);
  }
  uint4 *o = reinterpret_cast<uint4 *>(roots + 32 * j);
  o[0] = make_uint4(h[0], h[1], h[2], h[3]);
  o[1] = make_uint4(h[4], h[5], h[6], h[7]);
}

// The leader's root tree over {root, 0, ..., 0} of N parties: its root is
// log2(N) self-hashes of the party root (coPCS.cpp:193-201).
__global__ void party_root_kernel(const uint8_t *root, int logN, uint8_t *out, uint64_t root_stride) {
  if (threadIdx.x) return;
  root += root_stride * blockIdx.x;  // one CTA per party
  out += 32 * blockIdx.x;
  uint32_t m[16], h[8];
  for (int k = 0; k < 8; k++) h[k] = reinterpret_cast<const uint32_t *>(root)[k];
  for (int lv = 0; lv < logN; lv++) {
    for (int k = 0; k < 8; k++) { m[k] = h[k]; m[8 + k] = h[k]; }
    blake3_block64(m, h);
  }
  for (int k = 0; k < 8; k++) reinterpret_cast<uint32_t *>(out)[k] = h[k];
}

// Packed Shamir shares: group i of k secrets (plus _k - k random values)
// maps to party j's share by a fixed linear form mu[j][t].
__global__ void __launch_bounds__(256)
shares_kernel(const fe *v, const fe *fill, uint64_t groups, int N, int k, int kk, const fe *mu, fe *shares) {
  __shared__ fe smu[64 * 32];
  for (int t = threadIdx.x; t < N * kk; t += blockDim.x) smu[t] = mu[t];
  __syncthreads();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= groups) return;
  fe buf[32];
  for (int t = 0; t < k; t++) buf[t] = v[i * k + t];
  for (int t = k; t < kk; t++) buf[t] = fill ? fill[i * (kk - k) + (t - k)] : fe_zero();
  for (int j = 0; j < N; j++) {
    fe acc = fe_zero();
    for (int t = 0; t < kk; t++) acc = fadd(acc, fmul(smu[j * kk + t], buf[t]));
    shares[(uint64_t)j * groups + i] = acc;
  }
}

// out[i] = sum_p lambda_p msgs[p][i].  A CTA takes 32 consecutive
// coefficients (coalesced loads) and splits the parties over its 8 rows of
// threads (p = y mod 8), whose sums meet in shared memory: eight times the
// loads in flight of one thread per coefficient.
constexpr int kAggrCols = 32, kAggrRows = 8;
__global__ void __launch_bounds__(kAggrCols * kAggrRows)
aggregate_kernel(const fe *msgs, int N, uint64_t len, const fe *lambda, fe *out) {
  __shared__ fe red[kAggrRows][kAggrCols];
  const uint64_t i = (uint64_t)blockIdx.x * kAggrCols + threadIdx.x;
  fe acc = fe_zero();
  if (i < len)
    for (int p = threadIdx.y; p < N; p += kAggrRows) acc = fadd(acc, fmul(lambda[p], msgs[(uint64_t)p * len + i]));
  red[threadIdx.y][threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.y == 0 && i < len) {
    fe s = red[0][threadIdx.x];
    for (int y = 1; y < kAggrRows; y++) s = fadd(s, red[y][threadIdx.x]);
    out[i] = s;
  }
}

// The leader's unpack-and-weight map on the device (one CTA, N <= 1024): the
// form sum_{j < N/4} b_j E[2j] of the unpacked shares E = DFT(D IDFT(s)),
// D = diag(omega_{2N}^{-i}), is lambda^T s with lambda = IDFT(D DFT(g)),
// g[2j] = b_j (both transform matrices are symmetric).
constexpr int kLambdaMax = 1024;
__global__ void __launch_bounds__(1024) lambda_kernel(const fe *b, int N, int logN, fe *lambda) {
  __shared__ fe g[kLambdaMax], h[kLambdaMax], W[kLambdaMax];
  const int k = threadIdx.x;
  const fe w = root_of_unity(logN);
  if (k < N) {
    W[k] = fpow(w, (uint64_t)k);
    g[k] = ((k & 1) == 0 && (k >> 1) < N / 4) ? b[k >> 1] : fe_zero();
  }
  __syncthreads();
  if (k < N) {  // h = D DFT(g)
    fe acc = fe_zero();
    for (int j = 0; j < N; j += 2) acc = fadd(acc, fmul(g[j], W[(j * k) & (N - 1)]));
    h[k] = fmul(acc, fpow(finv(root_of_unity(logN + 1)), (uint64_t)k));
  }
  __syncthreads();
  if (k < N) {  // lambda = IDFT(h)
    fe acc = fe_zero();
    for (int j = 0; j < N; j++) acc = fadd(acc, fmul(h[j], W[(N - ((j * k) & (N - 1))) & (N - 1)]));
    lambda[k] = fmul(acc, finv(fe_make((uint64_t)N, 0)));
  }
}

// flags[blk] = 1 when block blk of v has a non-zero entry.
__global__ void nonzero_blocks_kernel(const fe *v, uint64_t nblocks, int logd, uint8_t *flags) {
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  const fe *p = v + (b << logd);
  uint8_t nz = 0;
  for (uint32_t k = 0; k < (1u << logd); k++) nz |= (p[k].re | p[k].im) ? 1 : 0;
  flags[b] = nz;
}

// Per-CTA partial sums of the extended-block products:
// quadratic: e1 * e2; cubic: (e1 * e2 - e4) * e3 over blocks with flags set.
// blockIdx.y selects a chunk of Dc = min(D, 256) positions k; within the
// CTA k = chunk * Dc + tid % Dc and lane = tid / Dc walks the blocks.
__global__ void __launch_bounds__(256)
cophase1_partial_kernel(const fe *e1, const fe *e2, const fe *e3, const fe *e4, const uint8_t *flags,
                        uint64_t nblocks, int logD, int blocks_per_cta, fe *partial) {
  __shared__ fe red[256];
  // grid.z: the party; its blocks and partials follow the previous party's
  const uint64_t pe = (uint64_t)blockIdx.z * (nblocks << logD);
  e1 += pe;
  e2 += pe;
  if (e3) e3 += pe;
  if (e4) e4 += pe;
  if (flags) flags += (uint64_t)blockIdx.z * nblocks;
  partial += (uint64_t)blockIdx.z * ((uint64_t)gridDim.x << logD);
  const int logDc = logD < 8 ? logD : 8;
  const uint32_t Dc = 1u << logDc, lane = threadIdx.x >> logDc, lanes = 256u >> logDc;
  const uint32_t k = blockIdx.y * Dc + (threadIdx.x & (Dc - 1));
  const uint64_t b0 = (uint64_t)blockIdx.x * blocks_per_cta;
  const uint64_t b1 = min(b0 + blocks_per_cta, nblocks);
  fe acc = fe_zero();
  for (uint64_t b = b0 + lane; b < b1; b += lanes) {
    if (flags && !flags[b]) continue;
    const uint64_t at = (b << logD) + k;
    fe t = fmul(e1[at], e2[at]);
    if (e3) t = fmul(fsub(t, e4[at]), e3[at]);
    acc = fadd(acc, t);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  if (lane == 0) {
    for (uint32_t l = 1; l < lanes; l++) acc = fadd(acc, red[threadIdx.x + (l << logDc)]);
    partial[((uint64_t)blockIdx.x << logD) + k] = acc;
  }
}

// H[z D + k] = sum_c partial[z][c][k]: one warp per coefficient k, its
// lanes over the partials (grid.y: the party).
__global__ void sum_partials_kernel(const fe *partial, uint64_t nparts, uint32_t D, fe *H) {
  const uint32_t k = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (k >= D) return;
  partial += (uint64_t)blockIdx.y * nparts * D;
  fe acc = fe_zero();
  for (uint64_t c = lane; c < nparts; c += 32) acc = fadd(acc, partial[c * D + k]);
  for (int d = 16; d > 0; d >>= 1) {
    fe t;
    t.re = __shfl_down_sync(0xffffffffu, acc.re, d);
    t.im = __shfl_down_sync(0xffffffffu, acc.im, d);
    acc = fadd(acc, t);
  }
  if (lane == 0) H[(uint64_t)blockIdx.y * D + k] = acc;
}

// coSumcheck phase 2: out[j] = sum_k L[k] v[j d + k].
__global__ void __launch_bounds__(256) cophase2_kernel(const fe *v, uint64_t nout, const fe *L, int logd, fe *out) {
  __shared__ fe sl[1024];
  const uint32_t d = 1u << logd;
  for (uint32_t k = threadIdx.x; k < d; k += blockDim.x) sl[k] = L[k];
  __syncthreads();
  const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nout) return;
  fe acc = fe_zero();
  for (uint32_t k = 0; k < d; k++) acc = fadd(acc, fmul(sl[k], v[(j << logd) + k]));
  out[j] = acc;
}

unsigned grid(uint64_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ------------------------------------------------------------ host side

// Naive DFT of length n over the host field code: out[k] = sum_j in[j] w^{jk}.
static std::vector<fe> host_dft(const std::vector<fe> &in, fe w) {
  const size_t n = in.size();
  std::vector<fe> out(n, fe_zero());
  fe wk = fe_one();
  for (size_t k = 0; k < n; k++) {
    fe x = fe_one(), acc = fe_zero();
    for (size_t j = 0; j < n; j++) {
      acc = fadd(acc, fmul(in[j], x));
      x = fmul(x, wk);
    }
    out[k] = acc;
    wk = fmul(wk, w);
  }
  return out;
}
static std::vector<fe> host_idft(const std::vector<fe> &in) {
  const int lg = ilog2(in.size());
  std::vector<fe> out = host_dft(in, finv(root_of_unity(lg)));
  const fe s = finv(fe_make(in.size(), 0));
  for (auto &x : out) x = fmul(x, s);
  return out;
}

std::vector<fe> shamir_share_matrix(int N) {
  // compute_secret_shares (MPI_utils.cpp:2747-2762): inverse transform of the
  // _k = N/2 group values, zero-pad to 2N, forward transform, party j takes
  // entry 2j+1.  Column t of the map is the image of the t-th unit vector.
  const int kk = N / 2;
  std::vector<fe> mu((size_t)N * kk);
  for (int t = 0; t < kk; t++) {
    std::vector<fe> e(kk, fe_zero());
    e[t] = fe_one();
    std::vector<fe> c = host_idft(e);
    c.resize(2 * N, fe_zero());
    std::vector<fe> ev = host_dft(c, root_of_unity(ilog2(2 * N)));
    for (int j = 0; j < N; j++) mu[(size_t)j * kk + t] = ev[2 * j + 1];
  }
  return mu;
}

std::vector<fe> aggregate_weights_even(int N, const std::vector<fe> &g) {
  // Per coefficient the N shares s are unpacked (unpack_secret_share with
  // _k = k = N, MPI_utils.cpp:2769-2785: E = DFT(D IDFT(s)), D =
  // diag(omega_{2N}^{-i})) and combined as g^T E.  Both transform matrices
  // are symmetric, so the weights of the shares are lambda = IDFT(D DFT(g)).
  const int lg = ilog2(N);
  std::vector<fe> h = host_dft(g, root_of_unity(lg));
  const fe w2n_inv = finv(root_of_unity(1 + lg));
  fe mul = fe_one();
  for (int i = 0; i < N; i++) {
    h[i] = fmul(mul, h[i]);
    mul = fmul(w2n_inv, mul);
  }
  return host_idft(h);
}

std::vector<fe> aggregate_weights(int N, const fe *b) {
  // sumcheck_aggr (MPI_utils.cpp:2631-2644): sum_{j < N/4} b_j E[2j], g[2j] = b_j.
  std::vector<fe> g(N, fe_zero());
  for (int j = 0; j < N / 4; j++) g[2 * j] = b[j];
  return aggregate_weights_even(N, g);
}

void multifold5_launch(const fe *cw, uint64_t n, const fe *a, int logd, fe *out, const NttTables &tn,
                       cudaStream_t s) {
  if (logd < 1 || logd > kMaxFoldLog) throw ArgError("RS_multifold5: fold degree must be 2..16");
  if (n < (2ull << logd)) throw ArgError("RS_multifold5: codeword shorter than two folds");
  const fe len_inv = finv(fe_make(1ull << logd, 0));
  FoldConsts k{};
  const fe om_inv = finv(root_of_unity(ilog2(n)));
  const uint64_t step = n >> logd;
  for (int lv = 0; lv < logd; lv++)
    for (int g = 0; g < (1 << (logd - 1 - lv)); g++) k.c[lv][g] = fpow(om_inv, ((uint64_t)g * step << lv) & (n - 1));
  const unsigned blocks = grid(n >> logd);
  switch (logd) {
    case 1: multifold5_kernel<1><<<blocks, 256, 0, s>>>(cw, n, a, out, tn.lo_inv, tn.hi_inv, len_inv, k); break;
    case 2: multifold5_kernel<2><<<blocks, 256, 0, s>>>(cw, n, a, out, tn.lo_inv, tn.hi_inv, len_inv, k); break;
    case 3: multifold5_kernel<3><<<blocks, 256, 0, s>>>(cw, n, a, out, tn.lo_inv, tn.hi_inv, len_inv, k); break;
    default: multifold5_kernel<4><<<blocks, 256, 0, s>>>(cw, n, a, out, tn.lo_inv, tn.hi_inv, len_inv, k); break;
  }
  GBZ_CUDA(cudaGetLastError());
}

void powers_launch(fe r, uint64_t n, fe *out, cudaStream_t s) {
  powers_kernel<<<grid(n), 256, 0, s>>>(r, n, out);
  GBZ_CUDA(cudaGetLastError());
}

namespace {
// out[r L + rate t + off] = x[r n + t]: a row's values at one residue of a
// codeword's positions.
__global__ void strided_copy_kernel(const fe *x, uint64_t n, fe *out, uint64_t L, int rate, int off) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  out[blockIdx.y * L + (uint64_t)rate * t + off] = x[blockIdx.y * n + t];
}
}  // namespace

void strided_copy_launch(const fe *x, uint64_t n, fe *out, uint64_t L, int rate, int off, int rows, cudaStream_t s) {
  if (rows < 1) return;
  if (rows > 65535) throw ArgError("strided copy: at most 65535 rows per launch");
  strided_copy_kernel<<<dim3(grid(n), (unsigned)rows), 256, 0, s>>>(x, n, out, L, rate, off);
  GBZ_CUDA(cudaGetLastError());
}

void coset_launch(fe *x, uint64_t n, const NttTables &t, cudaStream_t s, int rows, uint64_t row_stride) {
  if (rows < 1) return;
  coset_kernel<<<dim3(grid(n), (unsigned)rows), 256, 0, s>>>(x, n, t.lo_inv, t.hi_inv, row_stride);
  GBZ_CUDA(cudaGetLastError());
}

void column_merkle_launch(const fe *rows, int nrows, uint64_t L, uint8_t *levels, int logN, uint8_t *root,
                          cudaStream_t s, int parties, uint64_t rows_stride) {
  if (parties < 1 || parties > 65535) throw ArgError("column trees: 1..65535 parties per launch");
  const uint64_t tree = 32 * (2 * L - 1);
  column_root_kernel<<<dim3(grid(L), (unsigned)parties), 256, 0, s>>>(rows, nrows, L, levels, rows_stride, tree);
  GBZ_CUDA(cudaGetLastError());
  merkle_from_leaves_launch(levels, L, s, parties);
  party_root_kernel<<<parties, 32, 0, s>>>(levels + 32 * (2 * L - 2), logN, root, tree);
  GBZ_CUDA(cudaGetLastError());
}

void shares_launch(const fe *v, const fe *fill, uint64_t groups, int N, const fe *mu, fe *shares, cudaStream_t s) {
  shares_kernel<<<grid(groups), 256, 0, s>>>(v, fill, groups, N, N / 4, N / 2, mu, shares);
  GBZ_CUDA(cudaGetLastError());
}

void aggregate_weights_launch(const fe *b, int N, fe *lambda, cudaStream_t s) {
  if (N < 4 || N > kLambdaMax || (N & (N - 1))) throw ArgError("aggregate: N must be a power of two in [4, 1024]");
  lambda_kernel<<<1, N, 0, s>>>(b, N, ilog2((uint64_t)N), lambda);
  GBZ_CUDA(cudaGetLastError());
}

void aggregate_launch(const fe *msgs, int N, uint64_t len, const fe *lambda, fe *out, cudaStream_t s) {
  aggregate_kernel<<<(unsigned)((len + kAggrCols - 1) / kAggrCols), dim3(kAggrCols, kAggrRows), 0, s>>>(msgs, N, len,
                                                                                                 lambda, out);
  GBZ_CUDA(cudaGetLastError());
}

void nonzero_blocks_launch(const fe *v, uint64_t nblocks, int logd, uint8_t *flags, cudaStream_t s) {
  nonzero_blocks_kernel<<<grid(nblocks), 256, 0, s>>>(v, nblocks, logd, flags);
  GBZ_CUDA(cudaGetLastError());
}

uint64_t cophase1_parts(uint64_t nblocks, int blocks_per_cta) {
  return (nblocks + blocks_per_cta - 1) / blocks_per_cta;
}

void cophase1_reduce_launch(const fe *e1, const fe *e2, const fe *e3, const fe *e4, const uint8_t *flags,
                            uint64_t nblocks, int logD, int blocks_per_cta, fe *partial, fe *H, cudaStream_t s,
                            int parties) {
  if (logD > kMaxCoLogD) throw ArgError("coSumcheck: extended block longer than 2^13");
  if (parties < 1 || parties > 65535) throw ArgError("coSumcheck: 1..65535 parties per launch");
  const uint64_t parts = cophase1_parts(nblocks, blocks_per_cta);
  const unsigned chunks = logD > 8 ? 1u << (logD - 8) : 1u;
  cophase1_partial_kernel<<<dim3((unsigned)parts, chunks, (unsigned)parties), 256, 0, s>>>(
      e1, e2, e3, e4, flags, nblocks, logD, blocks_per_cta, partial);
  GBZ_CUDA(cudaGetLastError());
  sum_partials_kernel<<<dim3(grid(1ull << logD, 8), (unsigned)parties), 256, 0, s>>>(partial, parts, 1u << logD, H);
  GBZ_CUDA(cudaGetLastError());
}

void cophase2_launch(const fe *v, uint64_t n, const fe *L, int logd, fe *out, cudaStream_t s) {
  if (logd > 10) throw ArgError("coSumcheck phase 2: block longer than 1024");
  cophase2_kernel<<<grid(n >> logd), 256, 0, s>>>(v, n >> logd, L, logd, out);
  GBZ_CUDA(cudaGetLastError());
}

}  // namespace gbz
