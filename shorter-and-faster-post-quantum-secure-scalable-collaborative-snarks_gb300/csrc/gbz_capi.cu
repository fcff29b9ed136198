// extern "C" entry points of libgbz (declared in include/gbz.h).
#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <utility>

#include "../../include/gbz.h"
#include "gbz_ctx.cuh"
#include "gbz_batch_open.cuh"
#include "gbz_copcs.cuh"
#include "gbz_prover.cuh"
#include "gbz_rounds.cuh"
#include "gbz_sched.cuh"
#include "gbz_whir_aggr.cuh"

using namespace gbz;

using namespace gbz_api;

namespace {

__global__ void field_ops_kernel(const fe *a, const fe *b, uint64_t n, fe *s, fe *d, fe *p) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fe x = a[i], y = b[i];
  if (s) s[i] = fadd(x, y);
  if (d) d[i] = fsub(x, y);
  if (p) p[i] = fmul(x, y);
}

// comb_i = r^(i+1), omega_q[i] = omega_N^{q_i}.
__global__ void ub_prep_kernel(ProofState *st, const int32_t *q, int l, int logN, fe r) {
  if (threadIdx.x == 0) {
    fe c = r;
    for (int i = 0; i < l; i++) {
      st->comb[i] = c;
      c = fmul(c, r);
    }
  }
  // omega_N^q depends on q mod N only (N divides 2^32, so this also holds for
  // the reference's unsigned reading of a negative int).
  const fe om = root_of_unity(logN);
  const uint32_t mask = (1u << logN) - 1;
  for (int i = threadIdx.x; i < l; i += blockDim.x) {
    const uint32_t qr = (uint32_t)q[i] & mask;
    st->q[i] = (int32_t)qr;
    st->omega_q[i] = fpow(om, (uint64_t)qr);
  }
}

// Loads arbitrary weights: comb_i = c_i, q_i = q_i mod N, omega_q_i = omega_N^{q_i}.
__global__ void geo_prep_kernel(ProofState *st, const int32_t *q, const fe *c, int l, int logN) {
  const fe om = root_of_unity(logN);
  const uint32_t mask = (1u << logN) - 1;
  for (int i = threadIdx.x; i < l; i += blockDim.x) {
    const uint32_t qr = (uint32_t)q[i] & mask;
    st->q[i] = (int32_t)qr;
    st->comb[i] = c[i];
    st->omega_q[i] = fpow(om, (uint64_t)qr);
  }
}

}  // namespace

// b[j] += sum_i c_i omega_N^{q_i j} for j < nb (host q, c), in chunks of at
// most kMaxQueries terms, by the sparse transform or by direct sums.
static void geometric_update(gbz_ctx *ctx, fe *db, uint64_t nb, const int32_t *hq, const fe *hc, int l, int logN) {
  if (!ctx->st) GBZ_CUDA(cudaMalloc(&ctx->st, sizeof(ProofState)));
  if (!ctx->ub_scratch) GBZ_CUDA(cudaMalloc(&ctx->ub_scratch, sizeof(fe) * kUpdateBetasScratch));
  for (int i0 = 0; i0 < l; i0 += kMaxQueries) {
    const int cnt = std::min(kMaxQueries, l - i0);
    int32_t *dq = (int32_t *)ctx->buf(98, 4ull * kMaxQueries);
    fe *dc = (fe *)ctx->buf(99, 16ull * kMaxQueries);
    GBZ_CUDA(cudaMemcpyAsync(dq, hq + i0, 4ull * cnt, cudaMemcpyHostToDevice, ctx->stream));
    GBZ_CUDA(cudaMemcpyAsync(dc, hc + i0, 16ull * cnt, cudaMemcpyHostToDevice, ctx->stream));
    geo_prep_kernel<<<1, 256, 0, ctx->stream>>>(ctx->st, dq, dc, cnt, logN);
    GBZ_CUDA(cudaGetLastError());
    const uint64_t N = 1ull << logN;
    if (nb <= N && update_betas_by_transform(cnt, nb, N)) {
      fe *tmp = (fe *)ctx->buf(2, 16 * N);
      ntt_sparse_accumulate(ctx->tables(logN), ctx->st->q, ctx->st->comb, cnt, db, nb, tmp, ctx->stream);
    } else {
      update_betas_launch(db, nb, ctx->st, cnt, ctx->ub_scratch, ctx->stream);
    }
    GBZ_CUDA(cudaStreamSynchronize(ctx->stream));  // hq / hc chunks are host memory of the caller
  }
}

// The scale of tensor_eval_vector (coPCS.cpp:602-632) for party my_id:
// entry 2 my_id + 1 of the length-2N transform of the twice inversely
// transformed powers w2^t (t < cols, N = 2 cols).  Two inverse transforms of
// length n map x to x[(n - t) mod n] / n, so the entry is
// sum_t w2^{(cols - t) mod cols} / cols * omega_{2N}^{t (2 my_id + 1)}.
static fe tensor_scale(uint32_t p0, int cols, int my_id) {
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

static void check_tensor_shape(int cols, uint64_t rows, int rate, int my_id) {
  if (cols < 1 || cols > (1 << 20) || !is_pow2((uint64_t)cols)) throw ArgError("tensor: cols must be a power of two");
  if (my_id < 0 || my_id >= 2 * cols) throw ArgError("tensor: my_id must be below the number of parties");
  if (rate < 1 || !is_pow2((uint64_t)rate)) throw ArgError("tensor: rate must be a power of two");
  if (!is_pow2(rows) || ilog2(rows * (uint64_t)rate) > kMaxLogN)
    throw ArgError("tensor: rows * rate must be a power of two <= 2^28");
}

namespace gbz_api {

void encode_rows_device(gbz_ctx *ctx, const fe *drows, int nrows, int logrow, int rate, int log_rate_offset,
                        fe *dout) {
  const uint64_t n = 1ull << logrow, L = n * (uint64_t)rate;
  const NttTables &tn = ctx->tables(logrow), &tL = ctx->tables(ilog2(L));
  const NttTables &tw = ctx->tables(1 + log_rate_offset + logrow);
  // every row's inverse transform, coset shift and forward transform, the
  // rows side by side in each launch (chunks of up to 2^28 elements of
  // intermediate)
  const int chunk = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)nrows, (1ull << 28) / L));
  fe *tmp = (fe *)ctx->buf(2, 16 * L * (uint64_t)chunk);
  for (int r0 = 0; r0 < nrows; r0 += chunk) {
    const int rc = std::min(chunk, nrows - r0);
    fe *o = dout + L * (uint64_t)r0;
    const fe *x = drows + n * (uint64_t)r0;
    ntt_launch_rows(tn, x, n, n, o, L, rc, tmp, true, ctx->stream);
    coset_launch(o, n, tw, ctx->stream, rc, L);
    if (rate == 2 && log_rate_offset == 0 && n >= 2) {
      // The codeword is the interpolant P of the row on <w_n> evaluated at
      // w_2n^(m - 1): odd m give P(w_n^((m-1)/2)) = x[(m-1)/2], the row
      // itself, and even m the length-n transform of the shifted
      // coefficients (the same values as the zero-padded length-2n
      // transform, at half its cost).
      ntt_launch_rows(tn, o, n, L, o, L, rc, tmp, false, ctx->stream, 2);
      strided_copy_launch(x, n, o, L, 2, 1, rc, ctx->stream);
    } else {
      ntt_launch_rows(tL, o, n, L, o, L, rc, tmp, false, ctx->stream);
    }
  }
}

}  // namespace gbz_api

extern "C" {

gbz_status gbz_create(gbz_ctx **out, int device) {
  if (!out) return GBZ_EINVAL;
  *out = nullptr;
  gbz_ctx *ctx = new (std::nothrow) gbz_ctx();
  if (!ctx) return GBZ_ENOMEM;
  ctx->device = device;
  try {
    DeviceGuard g(device);
    GBZ_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->own_stream = true;
  } catch (const CudaError &e) {
    delete ctx;
    return GBZ_ECUDA;
  }
  *out = ctx;
  return GBZ_OK;
}

void gbz_destroy(gbz_ctx *ctx) {
  if (!ctx) return;
  try {
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->sched.reset();
    ctx->plans.clear();
    ctx->profilers.clear();
    for (auto &kv : ctx->ntt) ntt_tables_free(kv.second);
    for (auto &kv : ctx->scratch) cudaFree(kv.second.first);
    for (auto &kv : ctx->pools)
      for (auto &e : kv.second) cudaFree(e.first);
    cudaFree(ctx->st);
    cudaFree(ctx->ub_scratch);
    if (ctx->side.stream) {
      cudaStreamSynchronize(ctx->side.stream);
      cudaEventDestroy(ctx->side.fork);
      cudaEventDestroy(ctx->side.join);
      cudaStreamDestroy(ctx->side.stream);
    }
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  } catch (...) {
  }
  delete ctx;
}

gbz_status gbz_set_stream(gbz_ctx *ctx, void *stream) {
  API_BEGIN(ctx)
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ctx->own_stream) GBZ_CUDA(cudaStreamDestroy(ctx->stream));
  ctx->own_stream = false;
  ctx->stream = (cudaStream_t)stream;
  API_END(ctx)
}

void *gbz_get_stream(gbz_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

gbz_status gbz_synchronize(gbz_ctx *ctx) {
  API_BEGIN(ctx)
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END(ctx)
}

const char *gbz_status_string(gbz_status s) {
  switch (s) {
    case GBZ_OK: return "ok";
    case GBZ_EINVAL: return "invalid argument";
    case GBZ_ENOMEM: return "out of memory";
    case GBZ_ECUDA: return "CUDA error";
    case GBZ_ECHECK: return "device consistency check failed";
    case GBZ_ESMALL: return "output buffer too small";
    default: return "unknown status";
  }
}

const char *gbz_last_error(const gbz_ctx *ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

gbz_status gbz_host_alloc(void **ptr, uint64_t bytes) {
  if (!ptr) return GBZ_EINVAL;
  return cudaHostAlloc(ptr, bytes ? bytes : 16, cudaHostAllocDefault) == cudaSuccess ? GBZ_OK : GBZ_ENOMEM;
}
void gbz_host_free(void *ptr) {
  if (ptr) cudaFreeHost(ptr);
}
gbz_status gbz_device_alloc(gbz_ctx *ctx, void **ptr, uint64_t bytes) {
  API_BEGIN(ctx)
  need(ptr, "ptr");
  GBZ_CUDA(cudaMalloc(ptr, bytes ? bytes : 16));
  API_END(ctx)
}
void gbz_device_free(gbz_ctx *ctx, void *ptr) {
  if (!ctx || !ptr) return;
  try {
    DeviceGuard g(ctx->device);
    cudaFree(ptr);
  } catch (...) {
  }
}

gbz_status gbz_field_ops(gbz_ctx *ctx, const uint64_t *a, const uint64_t *b, uint64_t n, uint64_t *sum,
                         uint64_t *diff, uint64_t *prod, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(a, "a");
  need(b, "b");
  if (!n) return GBZ_OK;
  const uint64_t bytes = 16 * n;
  const fe *da = dev_view(ctx, 0, (const fe *)a, bytes, mem, true);
  const fe *db = dev_view(ctx, 1, (const fe *)b, bytes, mem, true);
  fe *ds = sum ? dev_view(ctx, 2, (fe *)sum, bytes, mem, false) : nullptr;
  fe *dd = diff ? dev_view(ctx, 3, (fe *)diff, bytes, mem, false) : nullptr;
  fe *dp = prod ? dev_view(ctx, 4, (fe *)prod, bytes, mem, false) : nullptr;
  field_ops_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(da, db, n, ds, dd, dp);
  GBZ_CUDA(cudaGetLastError());
  if (sum) copy_out(ctx, (fe *)sum, ds, bytes, mem);
  if (diff) copy_out(ctx, (fe *)diff, dd, bytes, mem);
  if (prod) copy_out(ctx, (fe *)prod, dp, bytes, mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_blake3_64(gbz_ctx *ctx, const uint8_t *in, uint8_t *out, uint64_t count, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(in, "in");
  need(out, "out");
  if (!count) return GBZ_OK;
  const uint8_t *din = dev_view(ctx, 0, in, 64 * count, mem, true);
  uint8_t *dout = dev_view(ctx, 1, out, 32 * count, mem, false);
  blake3_batch_launch(din, dout, count, ctx->stream);
  copy_out(ctx, out, dout, 32 * count, mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_fft(gbz_ctx *ctx, uint64_t *data, int logn, int inverse, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(data, "data");
  if (logn < 0 || logn > kMaxNttLogN) throw ArgError("fft: logn out of range [0, 26]");
  const uint64_t L = 1ull << logn, bytes = 16 * L;
  fe *d = dev_view(ctx, 0, (fe *)data, bytes, mem, true);
  fe *tmp = (fe *)ctx->buf(1, bytes);
  ntt_launch(ctx->tables(logn), d, L, d, tmp, inverse != 0, ctx->stream);
  copy_out(ctx, (fe *)data, d, bytes, mem);
  finish(ctx, mem);
  API_END(ctx)
}

// Reed-Solomon encoding of m coefficients into L = m * rate evaluations.
// Inputs in the base field take the half-length real-input transform; any
// other input (flagged on the device) the general one, with the same bytes.
static void rs_encode_launch(gbz_ctx *ctx, const fe *din, uint64_t m, uint64_t L, fe *dout, fe *tmp) {
  const bool overlap = (const void *)din < (const void *)(dout + L) && (const void *)dout < (const void *)(din + m);
  if (L < 4 || m < 2 || overlap) {
    ntt_launch(ctx->tables(ilog2(L)), din, m, dout, tmp, false, ctx->stream);
    return;
  }
  uint32_t *flag = (uint32_t *)ctx->buf(700, sizeof(uint32_t));
  GBZ_CUDA(cudaMemsetAsync(flag, 0, sizeof(uint32_t), ctx->stream));
  ntt_launch_real(ctx->tables(ilog2(L) - 1), ctx->tables(ilog2(L)), din, m, dout, tmp, flag, ctx->stream);
}

gbz_status gbz_rs_encode(gbz_ctx *ctx, const uint64_t *arr, uint64_t m, int rate, uint64_t *codeword, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(arr, "arr");
  need(codeword, "codeword");
  check_pow2(m, "rs_encode: m");
  if (rate < 1 || !is_pow2((uint64_t)rate)) throw ArgError("rs_encode: rate must be a power of two");
  const uint64_t L = m * (uint64_t)rate;
  if (ilog2(L) > kMaxNttLogN) throw ArgError("rs_encode: codeword longer than 2^26");
  const fe *din = dev_view(ctx, 0, (const fe *)arr, 16 * m, mem, true);
  fe *dout = dev_view(ctx, 1, (fe *)codeword, 16 * L, mem, false);
  fe *tmp = (fe *)ctx->buf(2, 16 * L);
  rs_encode_launch(ctx, din, m, L, dout, tmp);
  copy_out(ctx, (fe *)codeword, dout, 16 * L, mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_merkle_commit_blake(gbz_ctx *ctx, const uint64_t *elems, uint64_t N, uint8_t *levels, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(elems, "elems");
  need(levels, "levels");
  if (N < 4 || !is_pow2(N)) throw ArgError("merkle: N must be a power of two >= 4");
  const fe *d = dev_view(ctx, 0, (const fe *)elems, 16 * N, mem, true);
  uint8_t *lv = dev_view(ctx, 1, levels, 32 * merkle_hashes(N), mem, false);
  merkle_commit_launch(d, N, lv, ctx->stream);
  copy_out(ctx, levels, lv, 32 * merkle_hashes(N), mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_merkle_tree_from_leaves(gbz_ctx *ctx, const uint8_t *leaves, uint64_t L, uint8_t *levels, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(leaves, "leaves");
  need(levels, "levels");
  check_pow2(L, "create_tree_blake: leaf count");
  if (ilog2(L) > kMaxLogN) throw ArgError("create_tree_blake: more than 2^28 leaves");
  if (L == 1) return GBZ_OK;
  uint8_t *buf = (uint8_t *)ctx->buf(0, 32 * (2 * L - 1));
  const cudaMemcpyKind kin = mem == GBZ_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  GBZ_CUDA(cudaMemcpyAsync(buf, leaves, 32 * L, kin, ctx->stream));
  merkle_from_leaves_launch(buf, L, ctx->stream);
  const cudaMemcpyKind kout = mem == GBZ_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  GBZ_CUDA(cudaMemcpyAsync(levels, buf + 32 * L, 32 * (L - 1), kout, ctx->stream));
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_merkle_open_blake(const uint8_t *levels, uint64_t N, uint64_t pos, uint8_t *path, uint32_t *depth) {
  if (!levels || !path || N < 4 || !is_pow2(N)) return GBZ_EINVAL;
  uint64_t cnt = N / 4;
  if (pos >= cnt) return GBZ_EINVAL;
  const uint8_t *lv = levels;
  uint32_t d = 0;
  while (cnt > 1) {
    const uint64_t sib = 2 * (pos / 2) + (1 - (pos % 2));
    for (int k = 0; k < 32; k++) path[32 * d + k] = lv[32 * sib + k];
    d++;
    lv += 32 * cnt;
    cnt /= 2;
    pos /= 2;
  }
  if (depth) *depth = d;
  return GBZ_OK;
}

gbz_status gbz_whir_commit(gbz_ctx *ctx, const uint64_t *arr, uint64_t m, int rate, uint64_t *codeword,
                           uint8_t *levels, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(arr, "arr");
  need(codeword, "codeword");
  need(levels, "levels");
  check_pow2(m, "whir_commit: m");
  if (rate < 1 || !is_pow2((uint64_t)rate)) throw ArgError("whir_commit: rate must be a power of two");
  const uint64_t L = m * (uint64_t)rate;
  if (L < 4) throw ArgError("whir_commit: codeword shorter than one leaf");
  if (ilog2(L) > kMaxNttLogN) throw ArgError("whir_commit: codeword longer than 2^26");
  const fe *din = dev_view(ctx, 0, (const fe *)arr, 16 * m, mem, true);
  fe *dcw = dev_view(ctx, 1, (fe *)codeword, 16 * L, mem, false);
  uint8_t *dlv = dev_view(ctx, 2, levels, 32 * merkle_hashes(L), mem, false);
  fe *tmp = (fe *)ctx->buf(3, 16 * L);
  rs_encode_launch(ctx, din, m, L, dcw, tmp);
  merkle_commit_launch(dcw, L, dlv, ctx->stream);
  copy_out(ctx, (fe *)codeword, dcw, 16 * L, mem);
  copy_out(ctx, levels, dlv, 32 * merkle_hashes(L), mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_precompute_beta(gbz_ctx *ctx, const uint64_t *r, int nr, uint64_t *B, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(r, "r");
  need(B, "B");
  if (nr < 0 || nr > kMaxLogN) throw ArgError("precompute_beta: nr out of range [0, 28]");
  const fe *dr = dev_view(ctx, 0, (const fe *)r, 16 * (uint64_t)(nr ? nr : 1), mem, true);
  fe *dB = dev_view(ctx, 1, (fe *)B, 16ull << nr, mem, false);
  beta_launch(dr, nr, dB, ctx->stream);
  copy_out(ctx, (fe *)B, dB, 16ull << nr, mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_sumcheck_quadratic(gbz_ctx *ctx, const uint64_t *v1, const uint64_t *v2, uint64_t m,
                                  uint64_t *coeffs, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(v1, "v1");
  need(v2, "v2");
  need(coeffs, "coeffs");
  if (m < 2 || !is_pow2(m)) throw ArgError("sumcheck: m must be a power of two >= 2");
  const fe *a = dev_view(ctx, 0, (const fe *)v1, 16 * m, mem, true);
  const fe *b = dev_view(ctx, 1, (const fe *)v2, 16 * m, mem, true);
  const int blocks = sc_blocks(m / 2);
  fe *partial = (fe *)ctx->buf(2, 48ull * blocks);
  fe *out = (fe *)ctx->buf(3, 48);
  sc_step_launch(a, b, m, nullptr, nullptr, nullptr, true, partial, blocks, ctx->stream);
  sc_sum_launch(partial, blocks, out, ctx->stream);
  GBZ_CUDA(cudaMemcpyAsync(coeffs, out, 48, cudaMemcpyDeviceToHost, ctx->stream));
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END(ctx)
}

gbz_status gbz_sumcheck_fold(gbz_ctx *ctx, uint64_t *v, uint64_t m, const uint64_t *r, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(v, "v");
  need(r, "r");
  if (m < 2 || !is_pow2(m)) throw ArgError("sumcheck fold: m must be a power of two >= 2");
  fe *d = dev_view(ctx, 0, (fe *)v, 16 * m, mem, true);
  fe *dr = (fe *)ctx->buf(1, 16);
  GBZ_CUDA(cudaMemcpyAsync(dr, r, 16, cudaMemcpyHostToDevice, ctx->stream));
  fe *out = (fe *)ctx->buf(2, 8 * m);
  fe *out2 = (fe *)ctx->buf(3, 8 * m);
  // The fold kernel folds two vectors at once; the second one is a copy.
  sc_step_launch(d, d, m, dr, out, out2, false, nullptr, sc_blocks(m / 4 ? m / 4 : 1), ctx->stream);
  GBZ_CUDA(cudaMemcpyAsync(d, out, 8 * m, cudaMemcpyDeviceToDevice, ctx->stream));
  if (mem == GBZ_MEM_HOST) GBZ_CUDA(cudaMemcpyAsync(v, out, 8 * m, cudaMemcpyDeviceToHost, ctx->stream));
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_whir_update_betas(gbz_ctx *ctx, uint64_t *b, uint64_t nb, const int32_t *queries, int l, uint64_t N,
                                 const uint64_t *r, uint64_t *challenges, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(b, "b");
  need(r, "r");
  if (l < 0 || l > kMaxQueries) throw ArgError("update_betas: l out of range [0, 256]");
  if (l && !queries) throw ArgError("null pointer: queries");
  check_pow2(N, "update_betas: N");
  if (ilog2(N) > kMaxLogN) throw ArgError("update_betas: N above 2^28");
  if (!ctx->st) GBZ_CUDA(cudaMalloc(&ctx->st, sizeof(ProofState)));
  if (!ctx->ub_scratch) GBZ_CUDA(cudaMalloc(&ctx->ub_scratch, sizeof(fe) * kUpdateBetasScratch));
  fe *db = dev_view(ctx, 0, (fe *)b, 16 * nb, mem, true);
  const int32_t *dq = dev_view(ctx, 1, queries, 4ull * (l ? l : 1), mem, true);
  ub_prep_kernel<<<1, 256, 0, ctx->stream>>>(ctx->st, dq, l, ilog2(N), fe_make(r[0], r[1]));
  GBZ_CUDA(cudaGetLastError());
  if (nb == 0 || l == 0) {
    // nothing to update; the combination weights are still written
  } else if (update_betas_by_transform(l, nb, N)) {
    fe *tmp = (fe *)ctx->buf(2, 16 * N);
    ntt_sparse_accumulate(ctx->tables(ilog2(N)), ctx->st->q, ctx->st->comb, l, db, nb, tmp, ctx->stream);
  } else {
    update_betas_launch(db, nb, ctx->st, l, ctx->ub_scratch, ctx->stream);
  }
  copy_out(ctx, (fe *)b, db, 16 * nb, mem);
  if (challenges && l) {
    // challenges is host memory regardless of mem
    GBZ_CUDA(cudaMemcpyAsync(challenges, ctx->st->comb, 16ull * l, cudaMemcpyDeviceToHost, ctx->stream));
    GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  finish(ctx, mem);
  API_END(ctx)
}

void gbz_hash_to_field(uint64_t *state, const uint64_t *elems, int count, uint64_t *out) {
  fe s = fe_make(state[0], state[1]);
  for (int i = 0; i < count; i++) s = hash_F(s, fe_make(elems[2 * i], elems[2 * i + 1]));
  state[0] = s.re;
  state[1] = s.im;
  if (out) {
    out[0] = s.re;
    out[1] = s.im;
  }
}

static_assert(sizeof(gbz_prng) == sizeof(glibc_prng), "gbz_prng layout");

void gbz_prng_seed(gbz_prng *g, uint32_t seed) { prng_seed(*reinterpret_cast<glibc_prng *>(g), seed); }
int32_t gbz_prng_next(gbz_prng *g) { return prng_next(*reinterpret_cast<glibc_prng *>(g)); }
void gbz_prng_field(gbz_prng *g, uint64_t *out) {
  fe r = prng_field(*reinterpret_cast<glibc_prng *>(g));
  out[0] = r.re;
  out[1] = r.im;
}

void gbz_field_ops_host(const uint64_t *a, const uint64_t *b, uint64_t n, uint64_t *sum, uint64_t *diff,
                        uint64_t *prod) {
  for (uint64_t i = 0; i < n; i++) {
    fe x = fe_make(a[2 * i], a[2 * i + 1]), y = fe_make(b[2 * i], b[2 * i + 1]);
    if (sum) { fe r = fadd(x, y); sum[2 * i] = r.re; sum[2 * i + 1] = r.im; }
    if (diff) { fe r = fsub(x, y); diff[2 * i] = r.re; diff[2 * i + 1] = r.im; }
    if (prod) { fe r = fmul(x, y); prod[2 * i] = r.re; prod[2 * i + 1] = r.im; }
  }
}

int gbz_prove_launches(int logn, int rate) {
  try {
    if (logn < 3 || logn > 26 || rate < 2 || rate > 64 || !is_pow2((uint64_t)rate)) return 0;
    ProofPlan p;
    p.logn = logn;
    p.rate = rate;
    p.n = 1ull << logn;
    p.L = p.n * (uint64_t)rate;
    enqueue_proof(p, nullptr, 1, nullptr, true);
    return p.launches;
  } catch (...) {
    return 0;
  }
}

gbz_status gbz_set_graphs(gbz_ctx *ctx, int enable) {
  API_BEGIN(ctx)
  ctx->graphs = enable != 0;
  API_END(ctx)
}

gbz_status gbz_profile_enable(gbz_ctx *ctx, int enable) {
  API_BEGIN(ctx)
  ctx->profiling = enable != 0;
  API_END(ctx)
}

gbz_status gbz_profile_read(gbz_ctx *ctx, int logn, int rate, double *ms, int *groups) {
  API_BEGIN(ctx)
  need(ms, "ms");
  auto it = ctx->profilers.find(std::make_pair(logn, rate));
  if (it == ctx->profilers.end()) {
    for (int c = 0; c < PC_COUNT; c++) {
      ms[c] = 0;
      if (groups) groups[c] = 0;
    }
    return GBZ_OK;
  }
  it->second->read(ms, groups);
  it->second->reset();
  API_END(ctx)
}

gbz_status gbz_rs_multifold5(gbz_ctx *ctx, const uint64_t *cw, uint64_t n, const uint64_t *a, int logd, uint64_t *out,
                             int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(cw, "codeword");
  need(a, "a");
  need(out, "out");
  check_pow2(n, "RS_multifold5: n");
  if (ilog2(n) > kMaxLogN) throw ArgError("RS_multifold5: n above 2^28");
  const uint64_t d = 1ull << logd;
  const fe *dcw = dev_view(ctx, 0, (const fe *)cw, 16 * n, mem, true);
  fe *da = (fe *)ctx->buf(1, 16 * d * 2);
  GBZ_CUDA(cudaMemcpyAsync(da, a, 16 * d, cudaMemcpyHostToDevice, ctx->stream));
  fe *dout = dev_view(ctx, 2, (fe *)out, 16 * (n >> logd), mem, false);
  multifold5_launch(dcw, n, da, logd, dout, ctx->tables(ilog2(n)), ctx->stream);
  copy_out(ctx, (fe *)out, dout, 16 * (n >> logd), mem);
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END(ctx)
}

gbz_status gbz_lagrange_coeff(gbz_ctx *ctx, const uint64_t *r, int logd, uint64_t *out, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(r, "r");
  need(out, "out");
  if (logd < 0 || logd > 20) throw ArgError("lagrange: logd out of range [0, 20]");
  const uint64_t d = 1ull << logd;
  fe *dout = dev_view(ctx, 0, (fe *)out, 16 * d, mem, false);
  fe *tmp = (fe *)ctx->buf(1, 16 * d);
  powers_launch(fe_make(r[0], r[1]), d, dout, ctx->stream);
  ntt_launch(ctx->tables(logd), dout, d, dout, tmp, true, ctx->stream);
  copy_out(ctx, (fe *)out, dout, 16 * d, mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_encode_rows(gbz_ctx *ctx, const uint64_t *rows, int nrows, int logrow, int rate, int log_rate_offset,
                           uint64_t *out, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(rows, "rows");
  need(out, "out");
  if (nrows < 0 || logrow < 0 || log_rate_offset < 0) throw ArgError("encode: negative size");
  if (rate < 1 || !is_pow2((uint64_t)rate)) throw ArgError("encode: rate must be a power of two");
  const uint64_t n = 1ull << logrow, L = n * (uint64_t)rate;
  if (ilog2(L) > kMaxNttLogN || 1 + log_rate_offset + logrow > kMaxLogN) throw ArgError("encode: length above 2^26");
  if (!nrows) return GBZ_OK;
  const fe *drows = dev_view(ctx, 0, (const fe *)rows, 16 * n * nrows, mem, true);
  fe *dout = dev_view(ctx, 1, (fe *)out, 16 * L * nrows, mem, false);
  encode_rows_device(ctx, drows, nrows, logrow, rate, log_rate_offset, dout);
  copy_out(ctx, (fe *)out, dout, 16 * L * nrows, mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_encode_concatenated(gbz_ctx *ctx, const uint64_t *data, uint64_t n, int rate0, int rate1, int degree,
                                   uint64_t *Cprime, uint64_t *C, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(data, "data");
  need(C, "C");
  check_pow2(n, "encode_concatenated: n");
  if (rate0 < 1 || rate1 < 1 || !is_pow2((uint64_t)rate0) || !is_pow2((uint64_t)rate1))
    throw ArgError("encode_concatenated: rates must be powers of two");
  if (degree < 1 || !is_pow2((uint64_t)degree)) throw ArgError("encode_concatenated: degree must be a power of two");
  const uint64_t L = n * (uint64_t)rate0, D = (uint64_t)degree * rate1;
  if (ilog2(L) > kMaxNttLogN) throw ArgError("encode_concatenated: codeword above 2^26");
  if (D > (1u << 13)) throw ArgError("encode_concatenated: degree * rate1 above 2^13");
  if ((uint64_t)degree > L) throw ArgError("encode_concatenated: degree above the codeword length");
  const uint64_t rows = L / degree;
  const fe *din = dev_view(ctx, 0, (const fe *)data, 16 * n, mem, true);
  fe *dcp = (Cprime && mem == GBZ_MEM_DEVICE) ? (fe *)Cprime : (fe *)ctx->buf(1, 16 * L);
  fe *tmp = (fe *)ctx->buf(2, 16 * L);
  fe *dC = dev_view(ctx, 3, (fe *)C, 16 * rows * D, mem, false);
  ntt_launch(ctx->tables(ilog2(L)), din, n, dcp, tmp, false, ctx->stream);
  ntt_batched_strided(ctx->tables(ilog2(D)), dcp, rows, (uint32_t)degree, dC, rows, false, ctx->stream);
  if (Cprime && mem == GBZ_MEM_HOST) copy_out(ctx, (fe *)Cprime, dcp, 16 * L, mem);
  copy_out(ctx, (fe *)C, dC, 16 * rows * D, mem);
  finish(ctx, mem);
  API_END(ctx)
}

void gbz_leader_root(const uint8_t *root, int nparties, uint8_t *out) {
  uint32_t h[8], m[16];
  std::memcpy(h, root, 32);
  for (int n = nparties; n > 1; n /= 2) {
    for (int k = 0; k < 8; k++) m[k] = m[8 + k] = h[k];
    blake3_block64(m, h);
  }
  std::memcpy(out, h, 32);
}

gbz_status gbz_column_merkle(gbz_ctx *ctx, const uint64_t *rows, int nrows, int logL, int nparties, uint8_t *levels,
                             uint8_t *root, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(rows, "rows");
  need(levels, "levels");
  need(root, "root");
  if (nrows < 1 || nrows > 32) throw ArgError("column merkle: 1..32 rows");
  if (logL < 0 || logL > kMaxLogN) throw ArgError("column merkle: logL out of range");
  if (nparties < 1 || !is_pow2((uint64_t)nparties)) throw ArgError("column merkle: parties must be a power of two");
  const uint64_t L = 1ull << logL, nh = 2 * L - 1;
  const fe *drows = dev_view(ctx, 0, (const fe *)rows, 16 * L * nrows, mem, true);
  uint8_t *dlv = dev_view(ctx, 1, levels, 32 * nh, mem, false);
  uint8_t *droot = dev_view(ctx, 2, root, 32, mem, false);
  column_merkle_launch(drows, nrows, L, dlv, ilog2(nparties), droot, ctx->stream);
  copy_out(ctx, levels, dlv, 32 * nh, mem);
  copy_out(ctx, root, droot, 32, mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_secret_shares(gbz_ctx *ctx, const uint64_t *v, uint64_t M, int N, int privacy, uint32_t seed,
                             uint64_t *shares, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(v, "v");
  need(shares, "shares");
  if (N < 4 || N > 64 || !is_pow2((uint64_t)N)) throw ArgError("secret shares: N must be a power of two in [4, 64]");
  const int k = N / 4, kk = N / 2;
  if (M % (uint64_t)k) throw ArgError("secret shares: M must be a multiple of N/4");
  const uint64_t groups = M / k;
  const fe *dv = dev_view(ctx, 0, (const fe *)v, 16 * M, mem, true);
  fe *dsh = dev_view(ctx, 1, (fe *)shares, 16 * groups * N, mem, false);
  std::vector<fe> mu = shamir_share_matrix(N);
  fe *dmu = (fe *)ctx->buf(2, 16 * mu.size());
  GBZ_CUDA(cudaMemcpyAsync(dmu, mu.data(), 16 * mu.size(), cudaMemcpyHostToDevice, ctx->stream));
  fe *dfill = nullptr;
  std::vector<fe> fill;
  if (privacy) {  // F(random()) for the slots k.._k-1 of every group, in order
    glibc_prng g;
    prng_seed(g, seed);
    fill.resize(groups * (kk - k));
    for (auto &x : fill) x = fe_make((uint64_t)prng_next(g), 0);
    dfill = (fe *)ctx->buf(3, 16 * fill.size());
    GBZ_CUDA(cudaMemcpyAsync(dfill, fill.data(), 16 * fill.size(), cudaMemcpyHostToDevice, ctx->stream));
  }
  shares_launch(dv, dfill, groups, N, dmu, dsh, ctx->stream);
  copy_out(ctx, (fe *)shares, dsh, 16 * groups * N, mem);
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));  // host staging buffers above must outlive the copies
  API_END(ctx)
}

gbz_status gbz_party_aggregate(gbz_ctx *ctx, const uint64_t *msgs, int N, uint64_t len, const uint64_t *b,
                               uint64_t *out, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(msgs, "msgs");
  need(b, "b");
  need(out, "out");
  if (N < 4 || N > 1024 || !is_pow2((uint64_t)N)) throw ArgError("aggregate: N must be a power of two in [4, 1024]");
  const fe *dm = dev_view(ctx, 0, (const fe *)msgs, 16 * len * N, mem, true);
  // the unpack-and-weight map, built on the device from the N/4 weights (host memory)
  fe *db = (fe *)ctx->buf(3, 16ull * (N / 4));
  GBZ_CUDA(cudaMemcpyAsync(db, b, 16ull * (N / 4), cudaMemcpyHostToDevice, ctx->stream));
  fe *dl = (fe *)ctx->buf(1, 16 * N);
  aggregate_weights_launch(db, N, dl, ctx->stream);
  fe *dout = dev_view(ctx, 2, (fe *)out, 16 * len, mem, false);
  aggregate_launch(dm, N, len, dl, dout, ctx->stream);
  copy_out(ctx, (fe *)out, dout, 16 * len, mem);
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END(ctx)
}

gbz_status gbz_cosumcheck_phase1(gbz_ctx *ctx, const uint64_t *p1, const uint64_t *p2, const uint64_t *p3,
                                 const uint64_t *b1, uint64_t n, int logd, uint64_t *H, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(p1, "p1");
  need(p2, "p2");
  need(H, "H");
  const bool cubic = p3 || b1;
  if (cubic && !(p3 && b1)) throw ArgError("coSumcheck phase 1: the cubic form needs p3 and b1");
  const int ext = cubic ? 2 : 1, logD = logd + ext;
  if (logd < 0 || logD > kMaxCoLogD) throw ArgError("coSumcheck phase 1: extended block longer than 2^13");
  check_pow2(n, "coSumcheck phase 1: n");
  const uint64_t d = 1ull << logd, D = 1ull << logD;
  if (n < d) throw ArgError("coSumcheck phase 1: n below one block");
  const uint64_t nblocks = n / d;
  const fe *src[4] = {(const fe *)p1, (const fe *)p2, cubic ? (const fe *)b1 : nullptr,
                      cubic ? (const fe *)p3 : nullptr};
  const fe *dsrc[4] = {nullptr, nullptr, nullptr, nullptr};
  fe *ex[4] = {nullptr, nullptr, nullptr, nullptr};
  fe *coef = (fe *)ctx->buf(10, 16 * n);
  const NttTables &td = ctx->tables(logd), &tD = ctx->tables(logD);
  const int nv = cubic ? 4 : 2;
  for (int v = 0; v < nv; v++) {  // ext(v) per block: inverse of length d, forward of length D
    dsrc[v] = dev_view(ctx, 11 + v, src[v], 16 * n, mem, true);
    ex[v] = (fe *)ctx->buf(20 + v, 16 * nblocks * D);
    ntt_batched(td, dsrc[v], d, (uint32_t)d, coef, nblocks, true, ctx->stream);
    ntt_batched(tD, coef, d, (uint32_t)d, ex[v], nblocks, false, ctx->stream);
  }
  uint8_t *flags = nullptr;
  if (cubic) {  // blocks whose p1 part is all zero are skipped (coSumcheck.cpp:21-27)
    flags = (uint8_t *)ctx->buf(30, nblocks);
    nonzero_blocks_launch(dsrc[0], nblocks, logd, flags, ctx->stream);
  }
  const int lanes = D >= 256 ? 1 : (int)(256 / D);
  const int per_cta = (int)std::max<uint64_t>((uint64_t)lanes, (nblocks + 607) / 608);
  fe *partial = (fe *)ctx->buf(31, 16 * D * cophase1_parts(nblocks, per_cta));
  fe *dH = (fe *)ctx->buf(32, 16 * D);
  cophase1_reduce_launch(ex[0], ex[1], ex[2], ex[3], flags, nblocks, logD, per_cta, partial, dH, ctx->stream);
  GBZ_CUDA(cudaMemcpyAsync(H, dH, 16 * D, cudaMemcpyDeviceToHost, ctx->stream));
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END(ctx)
}

gbz_status gbz_cosumcheck_phase2(gbz_ctx *ctx, const uint64_t *v, uint64_t n, const uint64_t *L, int logd,
                                 uint64_t *out, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(v, "v");
  need(L, "L");
  need(out, "out");
  check_pow2(n, "coSumcheck phase 2: n");
  if (logd < 0 || logd > 10 || (n >> logd) == 0) throw ArgError("coSumcheck phase 2: block size out of range");
  const uint64_t d = 1ull << logd;
  const fe *dv = dev_view(ctx, 0, (const fe *)v, 16 * n, mem, true);
  fe *dL = (fe *)ctx->buf(1, 16 * d);
  GBZ_CUDA(cudaMemcpyAsync(dL, L, 16 * d, cudaMemcpyHostToDevice, ctx->stream));
  fe *dout = dev_view(ctx, 2, (fe *)out, 16 * (n >> logd), mem, false);
  cophase2_launch(dv, n, dL, logd, dout, ctx->stream);
  copy_out(ctx, (fe *)out, dout, 16 * (n >> logd), mem);
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END(ctx)
}

}  // extern "C"

namespace {

gbz_status prove_many(gbz_ctx *ctx, int count, const double *arrival_s, const uint64_t *const *witness,
                      const int *logn, const int *rate, const uint32_t *prng_seed, uint8_t *const *transcript,
                      const uint64_t *capacity, int mem, const gbz_sched_opts *opts, double *latency_s,
                      double *makespan_s) {
  API_BEGIN(ctx)
  check_mem(mem);
  if (count < 0) throw ArgError("count must be non-negative");
  if (count > 0) {
    need(witness, "witness");
    need(logn, "logn");
    need(rate, "rate");
    need(prng_seed, "prng_seed");
    need(transcript, "transcript");
    need(capacity, "capacity");
  }
  SchedOpts o;
  o.group = ctx->group;
  if (opts) {
    if (opts->lanes < 0 || opts->lanes > 64) throw ArgError("sched: lanes must be in [0, 64]");
    if (opts->depth < 0) throw ArgError("sched: depth must be non-negative");
    if (opts->lanes) o.lanes = opts->lanes;
    if (opts->depth) o.depth = opts->depth;
    if (opts->graphs >= 0) o.graphs = opts->graphs != 0;
    if (opts->reserve_bytes) o.reserve = opts->reserve_bytes;
  }
  std::vector<ProofJob> jobs(count);
  for (int i = 0; i < count; i++) {
    need(witness[i], "witness[i]");
    need(transcript[i], "transcript[i]");
    const uint64_t tb = gbz_prove_transcript_bytes(logn[i], rate[i]);
    if (!tb) throw ArgError("proof " + std::to_string(i) + ": unsupported shape 2^" + std::to_string(logn[i]) +
                            " at rate " + std::to_string(rate[i]));
    if (capacity[i] < tb)
      return fail(ctx, GBZ_ESMALL, "proof " + std::to_string(i) + ": transcript buffer smaller than gbz_prove_transcript_bytes");
    if (arrival_s && !(arrival_s[i] >= 0)) throw ArgError("arrival times must be non-negative");
    jobs[i].witness = (const fe *)witness[i];
    jobs[i].logn = logn[i];
    jobs[i].rate = rate[i];
    jobs[i].seed = prng_seed[i];
    jobs[i].transcript = transcript[i];
  }
  if (!ctx->sched) ctx->sched.reset(new Scheduler());
  std::vector<uint32_t> errors;
  ctx->sched->run(jobs, arrival_s, mem, o, latency_s, makespan_s, errors);
  for (int i = 0; i < count; i++)
    if (errors[i])
      return fail(ctx, GBZ_ECHECK, "proof " + std::to_string(i) + ": a sumcheck round message did not match its claim");
  API_END(ctx)
}

}  // namespace

extern "C" {

gbz_status gbz_prove_batch(gbz_ctx *ctx, int count, const uint64_t *const *witness, const int *logn, const int *rate,
                           const uint32_t *prng_seed, uint8_t *const *transcript, const uint64_t *capacity, int mem,
                           const gbz_sched_opts *opts, double *latency_s, double *makespan_s) {
  return prove_many(ctx, count, nullptr, witness, logn, rate, prng_seed, transcript, capacity, mem, opts, latency_s,
                    makespan_s);
}

gbz_status gbz_serve(gbz_ctx *ctx, int count, const double *arrival_s, const uint64_t *const *witness,
                     const int *logn, const int *rate, const uint32_t *prng_seed, uint8_t *const *transcript,
                     const uint64_t *capacity, int mem, const gbz_sched_opts *opts, double *latency_s,
                     double *makespan_s) {
  if (count > 0 && !arrival_s) {
    if (!ctx) return GBZ_EINVAL;
    return fail(ctx, GBZ_EINVAL, "null pointer: arrival_s");
  }
  return prove_many(ctx, count, arrival_s, witness, logn, rate, prng_seed, transcript, capacity, mem, opts,
                    latency_s, makespan_s);
}

gbz_status gbz_sched_set_grouping(gbz_ctx *ctx, int on) {
  if (!ctx) return GBZ_EINVAL;
  ctx->group = on != 0;
  return GBZ_OK;
}

gbz_status gbz_sched_release(gbz_ctx *ctx, uint64_t *cached_bytes) {
  API_BEGIN(ctx)
  uint64_t bytes = ctx->sched ? ctx->sched->cached_bytes() : 0;
  ctx->sched.reset();
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  for (auto &kv : ctx->pools)
    for (auto &e : kv.second) {
      bytes += e.second;
      cudaFree(e.first);
    }
  ctx->pools.clear();
  if (cached_bytes) *cached_bytes = bytes;
  API_END(ctx)
}

gbz_status gbz_sumcheck_round(gbz_ctx *ctx, int form, uint64_t *const *v, uint64_t m, const uint64_t *b,
                              const uint64_t *r, uint64_t *coeffs, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  const int nv = form_vectors(form), nc = form_coeffs(form);
  if (!nv) throw ArgError("sumcheck round: unknown form");
  need(v, "v");
  need(coeffs, "coeffs");
  if ((form == SC_BATCH || form == SC_ZEROCHECK) && !b) throw ArgError("sumcheck round: this form needs b");
  check_pow2(m, "sumcheck round: m");
  if (m < 2) throw ArgError("sumcheck round: m must be at least 2");
  RoundArgs a{};
  fe *scal = (fe *)ctx->buf(50, 16 * 2);
  fe hb[2] = {b ? fe_make(b[0], b[1]) : fe_zero(), r ? fe_make(r[0], r[1]) : fe_zero()};
  GBZ_CUDA(cudaMemcpyAsync(scal, hb, sizeof(hb), cudaMemcpyHostToDevice, ctx->stream));
  a.b = b ? scal : nullptr;
  a.r = scal + 1;
  fe *dv[6];
  for (int k = 0; k < nv; k++) {
    need(v[k], "v[k]");
    dv[k] = dev_view(ctx, 40 + k, (fe *)v[k], 16 * m, mem, true);
    a.in[k] = dv[k];
  }
  fe *dout = (fe *)ctx->buf(57, 16 * kMaxFormCoeffs);
  GBZ_CUDA(cudaMemsetAsync(dout, 0, 16 * kMaxFormCoeffs, ctx->stream));
  if (r) {
    const uint64_t half = m / 2;
    for (int k = 0; k < nv; k++) a.out[k] = (fe *)ctx->buf(60 + k, 16 * half);
    if (m >= 4) {
      a.pairs = m / 4;
      const int blocks = round_blocks(a.pairs);
      a.partial = (fe *)ctx->buf(56, 16 * kMaxFormCoeffs * (uint64_t)blocks);
      form_step_launch(form, a, 1, blocks, ctx->stream);
      form_sum_launch(a.partial, blocks, nc, dout, ctx->stream);
    } else {
      a.pairs = 1;  // the folded vectors have one entry: no pair, zero message
      form_step_launch(form, a, 2, 1, ctx->stream);
    }
    for (int k = 0; k < nv; k++)
      GBZ_CUDA(cudaMemcpyAsync(v[k], a.out[k], 16 * half,
                               mem == GBZ_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    a.pairs = m / 2;
    const int blocks = round_blocks(a.pairs);
    a.partial = (fe *)ctx->buf(56, 16 * kMaxFormCoeffs * (uint64_t)blocks);
    form_step_launch(form, a, 0, blocks, ctx->stream);
    form_sum_launch(a.partial, blocks, nc, dout, ctx->stream);
  }
  GBZ_CUDA(cudaMemcpyAsync(coeffs, dout, 16 * nc, cudaMemcpyDeviceToHost, ctx->stream));
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END(ctx)
}

namespace {
// Device views of count vectors of n elements (slots base..base+count-1).
VecList vec_views(gbz_ctx *ctx, int base, const uint64_t *const *v, int count, uint64_t n, int mem) {
  if (count < 0 || count > kMaxVecs) throw ArgError("at most 64 vectors");
  need(v, "vector list");
  VecList l{};
  for (int i = 0; i < count; i++) {
    need(v[i], "vector");
    l.p[i] = dev_view(ctx, base + i, (const fe *)v[i], 16 * n, mem, true);
  }
  return l;
}
fe host_fe(const uint64_t *p, int64_t i) { return fe_make(p[2 * i], p[2 * i + 1]); }
}  // namespace

gbz_status gbz_whir_aggregate_claims(gbz_ctx *ctx, int k, const uint64_t *const *arrays, uint64_t n, int c,
                                     const uint64_t *points, gbz_prng *prng, uint64_t *arr, uint64_t *b_aggr,
                                     uint64_t *K, uint64_t *challenges, uint64_t *sums, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(points, "points");
  need(prng, "prng");
  need(arr, "arr");
  need(b_aggr, "b_aggr");
  need(K, "K");
  need(challenges, "challenges");
  check_pow2(n, "aggregate_claims: n");
  const int lg = ilog2(n);
  if (lg > kMaxLogN) throw ArgError("aggregate_claims: n above 2^28");
  if (k < 1 || c < 1 || k > 64 || c > 64) throw ArgError("aggregate_claims: 1..64 arrays and claims");
  const VecList A = vec_views(ctx, 100, arrays, k, n, mem);
  fe *dpts = (fe *)ctx->buf(90, 16 * (uint64_t)c * std::max(lg, 1));
  GBZ_CUDA(cudaMemcpyAsync(dpts, points, 16 * (uint64_t)c * lg, cudaMemcpyHostToDevice, ctx->stream));
  if (k <= 4 && c <= 4 && lg >= 2) {
    // one pass: the verifier's weights do not depend on the sums (they are
    // glibc draws), so they are drawn first and the pass forms the sums,
    // b_aggr and arr together from half-length eq tables
    glibc_prng g;
    std::memcpy(&g, prng, sizeof(g));
    std::vector<fe> ch(c + k);
    for (auto &x : ch) x = prng_field(g);
    std::memcpy(prng, &g, sizeof(g));
    fe *dch = (fe *)ctx->buf(94, 16 * (uint64_t)(c + k));
    GBZ_CUDA(cudaMemcpyAsync(dch, ch.data(), 16 * ch.size(), cudaMemcpyHostToDevice, ctx->stream));
    const int h = lg / 2;
    const uint64_t nlo = 1ull << h, nhi = 1ull << (lg - h);
    fe *elo = (fe *)ctx->buf(97, 16 * nlo * c), *ehi = (fe *)ctx->buf(98, 16 * nhi * c);
    for (int j = 0; j < c; j++) {
      beta_launch(dpts + (uint64_t)j * lg, h, elo + (uint64_t)j * nlo, ctx->stream);
      beta_launch(dpts + (uint64_t)j * lg + h, lg - h, ehi + (uint64_t)j * nhi, ctx->stream);
    }
    fe *partial = (fe *)ctx->buf(92, 16 * multidot_scratch(n));
    fe *dsums = (fe *)ctx->buf(93, 16 * (uint64_t)k * c);
    fe *dba = dev_view(ctx, 95, (fe *)b_aggr, 16 * n, mem, false);
    fe *darr = dev_view(ctx, 96, (fe *)arr, 16 * n, mem, false);
    aggr_claims_fused(A, k, c, elo, ehi, h, lg, n, dch, darr, dba, partial, dsums, ctx->stream);
    std::vector<fe> hs((size_t)k * c);
    GBZ_CUDA(cudaMemcpyAsync(hs.data(), dsums, 16 * hs.size(), cudaMemcpyDeviceToHost, ctx->stream));
    copy_out(ctx, (fe *)b_aggr, dba, 16 * n, mem);
    copy_out(ctx, (fe *)arr, darr, 16 * n, mem);
    GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
    fe Kacc = fe_zero();
    for (int i = 0; i < k; i++)
      for (int j = 0; j < c; j++) Kacc = fadd(Kacc, fmul(fmul(ch[j], ch[c + i]), hs[(size_t)i * c + j]));
    K[0] = Kacc.re;
    K[1] = Kacc.im;
    for (int i = 0; i < c + k; i++) {
      challenges[2 * i] = ch[i].re;
      challenges[2 * i + 1] = ch[i].im;
    }
    if (sums)
      for (size_t q = 0; q < hs.size(); q++) {
        sums[2 * q] = hs[q].re;
        sums[2 * q + 1] = hs[q].im;
      }
    return GBZ_OK;
  }
  fe *betas = (fe *)ctx->buf(91, 16 * n * (uint64_t)c);
  VecList Bt{};
  for (int j = 0; j < c; j++) {
    beta_launch(dpts + (uint64_t)j * lg, lg, betas + (uint64_t)j * n, ctx->stream);
    Bt.p[j] = betas + (uint64_t)j * n;
  }
  fe *partial = (fe *)ctx->buf(92, 16 * multidot_scratch(n));
  fe *dsums = (fe *)ctx->buf(93, 16 * (uint64_t)k * c);
  multidot_launch(A, k, Bt, c, n, partial, dsums, ctx->stream);
  std::vector<fe> hs((size_t)k * c);
  GBZ_CUDA(cudaMemcpyAsync(hs.data(), dsums, 16 * hs.size(), cudaMemcpyDeviceToHost, ctx->stream));
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  // verifier challenges: c beta weights, then k array weights (Whir.cpp:636-641)
  glibc_prng g;
  std::memcpy(&g, prng, sizeof(g));
  std::vector<fe> ch(c + k);
  for (auto &x : ch) x = prng_field(g);
  std::memcpy(prng, &g, sizeof(g));
  fe Kacc = fe_zero();
  for (int i = 0; i < k; i++)
    for (int j = 0; j < c; j++) Kacc = fadd(Kacc, fmul(fmul(ch[j], ch[c + i]), hs[(size_t)i * c + j]));
  K[0] = Kacc.re;
  K[1] = Kacc.im;
  for (int i = 0; i < c + k; i++) {
    challenges[2 * i] = ch[i].re;
    challenges[2 * i + 1] = ch[i].im;
  }
  if (sums)
    for (size_t q = 0; q < hs.size(); q++) {
      sums[2 * q] = hs[q].re;
      sums[2 * q + 1] = hs[q].im;
    }
  fe *dch = (fe *)ctx->buf(94, 16 * (uint64_t)(c + k));
  GBZ_CUDA(cudaMemcpyAsync(dch, ch.data(), 16 * ch.size(), cudaMemcpyHostToDevice, ctx->stream));
  fe *dba = dev_view(ctx, 95, (fe *)b_aggr, 16 * n, mem, false);
  fe *darr = dev_view(ctx, 96, (fe *)arr, 16 * n, mem, false);
  lincomb_launch(Bt, dch, c, n, dba, false, ctx->stream);
  lincomb_launch(A, dch + c, k, n, darr, false, ctx->stream);
  copy_out(ctx, (fe *)b_aggr, dba, 16 * n, mem);
  copy_out(ctx, (fe *)arr, darr, 16 * n, mem);
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));  // ch is a host temporary
  API_END(ctx)
}

gbz_status gbz_whir_aggregate_arrays(gbz_ctx *ctx, int k, const uint64_t *const *arrays, int nB,
                                     const uint64_t *const *B, uint64_t n, const uint64_t *r1, const uint64_t *r2,
                                     uint64_t *arr, uint64_t *b, uint64_t *K, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(r1, "r1");
  need(r2, "r2");
  need(arr, "arr");
  need(b, "b");
  need(K, "K");
  if (k < 1 || nB < k || nB > 64) throw ArgError("aggregate_arrays: 1 <= k <= nB <= 64");
  if (!n) throw ArgError("aggregate_arrays: empty arrays");
  const VecList A = vec_views(ctx, 100, arrays, k, n, mem);
  const VecList Bv = vec_views(ctx, 170, B, nB, n, mem);
  fe *partial = (fe *)ctx->buf(92, 16 * multidot_scratch(n));
  fe *dev = (fe *)ctx->buf(93, 16 * (uint64_t)k * nB);
  multidot_launch(A, k, Bv, nB, n, partial, dev, ctx->stream);
  std::vector<fe> ev((size_t)k * nB);
  GBZ_CUDA(cudaMemcpyAsync(ev.data(), dev, 16 * ev.size(), cudaMemcpyDeviceToHost, ctx->stream));
  // arr += sum_{i>=1} r1_i arrays_i, b += sum_{i>=1} r2_i B_i (Whir.cpp:689-694)
  std::vector<fe> coef(2 * (size_t)k);
  for (int i = 0; i < k; i++) {
    coef[i] = i ? host_fe(r1, i) : fe_zero();
    coef[k + i] = i ? host_fe(r2, i) : fe_zero();
  }
  fe *dcoef = (fe *)ctx->buf(94, 16 * coef.size());
  GBZ_CUDA(cudaMemcpyAsync(dcoef, coef.data(), 16 * coef.size(), cudaMemcpyHostToDevice, ctx->stream));
  fe *darr = dev_view(ctx, 96, (fe *)arr, 16 * n, mem, true);
  fe *db = dev_view(ctx, 95, (fe *)b, 16 * n, mem, true);
  lincomb_launch(A, dcoef, k, n, darr, true, ctx->stream);
  lincomb_launch(Bv, dcoef + k, k, n, db, true, ctx->stream);
  copy_out(ctx, (fe *)arr, darr, 16 * n, mem);
  copy_out(ctx, (fe *)b, db, 16 * n, mem);
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  fe Kacc = fe_zero();
  for (int i = 0; i < k; i++)
    for (int j = 0; j < nB; j++)
      Kacc = fadd(Kacc, fmul(fmul(host_fe(r1, i), host_fe(r2, j)), ev[(size_t)i * nB + j]));
  K[0] = Kacc.re;
  K[1] = Kacc.im;
  API_END(ctx)
}

gbz_status gbz_whir_aggregate_commitments(gbz_ctx *ctx, int k, const uint64_t *const *codewords, uint64_t n,
                                          const uint64_t *r, int rate, int whir_k, gbz_prng *prng,
                                          uint64_t *codeword, uint8_t *levels, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(r, "r");
  need(prng, "prng");
  need(codeword, "codeword");
  need(levels, "levels");
  if (k < 1 || k > 64) throw ArgError("aggregate_commitments: 1..64 codewords");
  if (whir_k < 4 || !is_pow2((uint64_t)whir_k)) throw ArgError("aggregate_commitments: whir_k must be a power of two >= 4");
  if (rate < 1) throw ArgError("aggregate_commitments: rate must be positive");
  check_pow2(n, "aggregate_commitments: n");
  if (n < (uint64_t)whir_k) throw ArgError("aggregate_commitments: codeword shorter than whir_k");
  const VecList C = vec_views(ctx, 100, codewords, k, n, mem);
  std::vector<fe> coef(k);
  for (int i = 0; i < k; i++) coef[i] = host_fe(r, i);
  fe *dcoef = (fe *)ctx->buf(94, 16 * coef.size());
  GBZ_CUDA(cudaMemcpyAsync(dcoef, coef.data(), 16 * coef.size(), cudaMemcpyHostToDevice, ctx->stream));
  fe *dcw = dev_view(ctx, 96, (fe *)codeword, 16 * n, mem, false);
  lincomb_launch(C, dcoef, k, n, dcw, false, ctx->stream);
  // query openings draw l values from rand() (Whir.cpp:574-576)
  glibc_prng g;
  std::memcpy(&g, prng, sizeof(g));
  const int l = whir_query_count(rate);
  for (int i = 0; i < l; i++) (void)prng_next(g);
  std::memcpy(prng, &g, sizeof(g));
  // the new tree over n / whir_k leaf hashes that the reference leaves zero (Whir.cpp:594-604)
  const uint64_t leaves = n / whir_k, nh = 2 * leaves - 1;
  uint8_t *dlv = dev_view(ctx, 97, levels, 32 * nh, mem, false);
  GBZ_CUDA(cudaMemsetAsync(dlv, 0, 32 * leaves, ctx->stream));
  merkle_from_leaves_launch(dlv, leaves, ctx->stream);
  copy_out(ctx, (fe *)codeword, dcw, 16 * n, mem);
  copy_out(ctx, levels, dlv, 32 * nh, mem);
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  API_END(ctx)
}

gbz_status gbz_whir_batch_schedule(int k, const uint64_t *sizes, int rate, int whir_k, int *steps, int32_t *kappa,
                                   int32_t *aggr, uint64_t *cw_len, uint64_t *transcript_bytes) {
  try {
    const BatchPlan P = batch_plan(k, sizes, rate, whir_k);
    if (steps) *steps = (int)P.kappa.size();
    for (size_t i = 0; i < P.kappa.size(); i++) {
      if (kappa) kappa[i] = P.kappa[i];
      if (aggr) aggr[i] = P.aggr[i];
    }
    if (cw_len)
      for (int i = 0; i < k; i++) cw_len[i] = P.cw_len[i];
    if (transcript_bytes) *transcript_bytes = P.transcript_bytes;
  } catch (const ArgError &) {
    return GBZ_EINVAL;
  }
  return GBZ_OK;
}

gbz_status gbz_whir_batch_open(gbz_ctx *ctx, int k, const uint64_t *const *arrays, const uint64_t *sizes,
                               const uint64_t *const *codewords, const uint8_t *levels0,
                               const uint64_t *const *betas, const uint64_t *K0, int rate, int whir_k,
                               gbz_prng *prng, uint8_t *transcript, uint64_t capacity, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(arrays, "arrays");
  need(codewords, "codewords");
  need(betas, "betas");
  need(levels0, "levels0");
  need(K0, "K0");
  need(prng, "prng");
  need(transcript, "transcript");
  const BatchPlan P = batch_plan(k, sizes, rate, whir_k);
  if (capacity < P.transcript_bytes) throw ArgError("transcript capacity below gbz_whir_batch_schedule's size");
  std::vector<const fe *> da(k, nullptr), db(k, nullptr), dc(k, nullptr);
  for (int i = 0; i < k; i++) {
    if (i && !P.cw_len[i]) continue;  // never merged: not read
    need(arrays[i], "arrays[i]");
    need(betas[i], "betas[i]");
    need(codewords[i], "codewords[i]");
    da[i] = dev_view(ctx, 400 + i, (const fe *)arrays[i], 16 * P.sizes[i], mem, true);
    db[i] = dev_view(ctx, 470 + i, (const fe *)betas[i], 16 * P.sizes[i], mem, true);
    dc[i] = dev_view(ctx, 540 + i, (const fe *)codewords[i], 16 * P.cw_len[i], mem, true);
  }
  const uint64_t L0 = P.cw_len[0];
  const uint8_t *dlv = dev_view(ctx, 610, levels0, 32 * merkle_hashes(L0), mem, true);
  if (!ctx->st) GBZ_CUDA(cudaMalloc(&ctx->st, sizeof(ProofState)));
  if (!ctx->ub_scratch) GBZ_CUDA(cudaMalloc(&ctx->ub_scratch, sizeof(fe) * kUpdateBetasScratch));
  uint8_t *dtr = mem == GBZ_MEM_DEVICE ? transcript : (uint8_t *)ctx->buf(620, P.transcript_bytes);
  BatchResources R;
  R.s = ctx->stream;
  R.buf = [ctx](int slot, uint64_t bytes) { return ctx->buf(slot, bytes); };
  R.tables = [ctx](int lg) -> NttTables & { return ctx->tables(lg); };
  R.st = ctx->st;
  R.ub_scratch = ctx->ub_scratch;
  glibc_prng g;
  static_assert(sizeof(g) == sizeof(gbz_prng), "generator state layout");
  std::memcpy(&g, prng, sizeof(g));
  batch_open_enqueue(R, P, da.data(), db.data(), dc.data(), dlv, fe_make(K0[0], K0[1]), g, dtr);
  copy_out(ctx, transcript, dtr, P.transcript_bytes, mem);
  uint32_t err = 0;
  GBZ_CUDA(cudaMemcpyAsync(&g, &ctx->st->prng, sizeof(g), cudaMemcpyDeviceToHost, ctx->stream));
  GBZ_CUDA(cudaMemcpyAsync(&err, &ctx->st->error, 4, cudaMemcpyDeviceToHost, ctx->stream));
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(prng, &g, sizeof(g));
  if (err) return fail(ctx, GBZ_ECHECK, "batch open: a device-side consistency check failed (flags " +
                                         std::to_string(err) + ")");
  API_END(ctx)
}

gbz_status gbz_tensor_eval_vector(gbz_ctx *ctx, const uint32_t *point, int cols, uint64_t rows, int rate, int my_id,
                                  uint64_t *out, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(point, "point");
  need(out, "out");
  check_tensor_shape(cols, rows, rate, my_id);
  fe *dout = dev_view(ctx, 0, (fe *)out, 16 * rows, mem, false);
  GBZ_CUDA(cudaMemsetAsync(dout, 0, 16 * rows, ctx->stream));
  const int32_t q = (int32_t)point[1];
  const fe c = tensor_scale(point[0], cols, my_id);
  geometric_update(ctx, dout, rows, &q, &c, 1, ilog2(rows * (uint64_t)rate));
  copy_out(ctx, (fe *)out, dout, 16 * rows, mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_pcs_sumcheck_phase3(gbz_ctx *ctx, uint64_t *B, uint64_t rows, const uint32_t *queries, int l,
                                   const uint64_t *s, int N, int rate, int my_id, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(B, "B");
  need(s, "s");
  if (l < 0) throw ArgError("phase 3: negative query count");
  if (l && !queries) throw ArgError("null pointer: queries");
  if (N < 2) throw ArgError("phase 3: at least two parties");
  check_tensor_shape(N / 2, rows, rate, my_id);
  std::vector<int32_t> q(l);
  std::vector<fe> c(l);
  const fe sv = fe_make(s[0], s[1]);
  fe p = sv;
  for (int i = 0; i < l; i++) {
    q[i] = (int32_t)queries[2 * i + 1];
    c[i] = fmul(p, tensor_scale(queries[2 * i], N / 2, my_id));
    p = fmul(p, sv);
  }
  fe *dB = dev_view(ctx, 0, (fe *)B, 16 * rows, mem, true);
  if (l) geometric_update(ctx, dB, rows, q.data(), c.data(), l, ilog2(rows * (uint64_t)rate));
  copy_out(ctx, (fe *)B, dB, 16 * rows, mem);
  finish(ctx, mem);
  API_END(ctx)
}

gbz_status gbz_ntt_set_shape(int logn, int k1, int log_cols_a, int log_rows_b) {
  try {
    ntt_set_shape(logn, NttShape{k1, log_cols_a, log_rows_b});
  } catch (const ArgError &) {
    return GBZ_EINVAL;
  }
  return GBZ_OK;
}

gbz_status gbz_ntt_get_shape(int logn, int *shape) {
  if (!shape) return GBZ_EINVAL;
  const NttShape sh = ntt_get_shape(logn);
  shape[0] = sh.k1;
  shape[1] = sh.logBA;
  shape[2] = sh.logBB;
  return sh.k1 > 0 ? GBZ_OK : GBZ_EINVAL;
}

void gbz_ntt_full_twiddles(int enable) { ntt_use_full_twiddles(enable != 0); }

gbz_status gbz_merkle_set_fusion(int log_nodes_per_cta) {
  try {
    merkle_set_fusion(log_nodes_per_cta);
  } catch (const ArgError &) {
    return GBZ_EINVAL;
  }
  return GBZ_OK;
}

int gbz_merkle_get_fusion(void) { return merkle_get_fusion(); }

gbz_status gbz_merkle_autotune(gbz_ctx *ctx, int logN, int reps, int *log_nodes, double *ms_default,
                               double *ms_best) {
  API_BEGIN(ctx)
  if (logN < 2 || logN > kMaxLogN) throw ArgError("merkle autotune: logN out of range [2, 28]");
  if (reps < 1) reps = 3;
  const uint64_t N = 1ull << logN;
  fe *elems = (fe *)ctx->buf(110, 16 * N);
  uint8_t *lv = (uint8_t *)ctx->buf(111, 32 * merkle_hashes(N));
  GBZ_CUDA(cudaMemsetAsync(elems, 0x11, 16 * N, ctx->stream));
  cudaEvent_t a, b;
  GBZ_CUDA(cudaEventCreate(&a));
  GBZ_CUDA(cudaEventCreate(&b));
  const int before = merkle_get_fusion();
  double best_ms = 1e30, def_ms = 0;
  int best = 10;
  for (int lg : {10, 11}) {
    merkle_set_fusion(lg);
    merkle_commit_launch(elems, N, lv, ctx->stream);
    double t = 1e30;
    for (int r = 0; r < reps; r++) {
      GBZ_CUDA(cudaEventRecord(a, ctx->stream));
      merkle_commit_launch(elems, N, lv, ctx->stream);
      GBZ_CUDA(cudaEventRecord(b, ctx->stream));
      GBZ_CUDA(cudaEventSynchronize(b));
      float ms = 0;
      GBZ_CUDA(cudaEventElapsedTime(&ms, a, b));
      t = std::min(t, (double)ms);
    }
    if (lg == 10) def_ms = t;
    if (t < best_ms) {
      best_ms = t;
      best = lg;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  (void)before;
  merkle_set_fusion(best);
  if (log_nodes) *log_nodes = best;
  if (ms_default) *ms_default = def_ms;
  if (ms_best) *ms_best = best_ms;
  API_END(ctx)
}

gbz_status gbz_ntt_autotune(gbz_ctx *ctx, int logn, int reps, int *shape, double *ms_default, double *ms_best) {
  API_BEGIN(ctx)
  if (logn <= 13 || logn > kMaxNttLogN) throw ArgError("ntt autotune: lengths 2^14 .. 2^26 (one pass below)");
  if (reps < 1) reps = 3;
  const uint64_t L = 1ull << logn;
  fe *buf = (fe *)ctx->buf(110, 16 * L);
  fe *tmp = (fe *)ctx->buf(111, 16 * L);
  GBZ_CUDA(cudaMemsetAsync(buf, 0x11, 16 * L, ctx->stream));  // any canonical-looking data; timing only
  const NttTables &t = ctx->tables(logn);
  const NttShape before = ntt_get_shape(logn);
  const NttShape dflt = ntt_default_shape(logn);
  cudaEvent_t a, b;
  GBZ_CUDA(cudaEventCreate(&a));
  GBZ_CUDA(cudaEventCreate(&b));
  auto time_shape = [&](const NttShape &sh) {
    ntt_set_shape(logn, sh);
    ntt_launch(t, buf, L, buf, tmp, false, ctx->stream);  // warm-up
    double best = 1e30;
    for (int r = 0; r < reps; r++) {
      GBZ_CUDA(cudaEventRecord(a, ctx->stream));
      ntt_launch(t, buf, L, buf, tmp, false, ctx->stream);
      GBZ_CUDA(cudaEventRecord(b, ctx->stream));
      GBZ_CUDA(cudaEventSynchronize(b));
      float ms = 0;
      GBZ_CUDA(cudaEventElapsedTime(&ms, a, b));
      best = std::min(best, (double)ms);
    }
    return best;
  };
  NttShape best_sh = dflt;
  double best_ms = 0, def_ms = 0;
  try {
    def_ms = best_ms = time_shape(dflt);
    for (const NttShape &sh : ntt_shape_candidates(logn)) {
      const double ms = time_shape(sh);
      if (ms < best_ms * 0.98) {  // keep the default unless clearly faster
        best_ms = ms;
        best_sh = sh;
      }
    }
  } catch (...) {
    ntt_set_shape(logn, before);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    throw;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  ntt_set_shape(logn, best_sh);
  outer_table_keep_only(logn, best_sh.k1);
  if (shape) {
    shape[0] = best_sh.k1;
    shape[1] = best_sh.logBA;
    shape[2] = best_sh.logBB;
  }
  if (ms_default) *ms_default = def_ms;
  if (ms_best) *ms_best = best_ms;
  API_END(ctx)
}

gbz_status gbz_calibrate(gbz_ctx *ctx, double *fmul_per_s, double *blake3_per_s) {
  API_BEGIN(ctx)
  int sms = 0;
  GBZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  void *scratch = ctx->buf(48, calibrate_scratch_bytes(sms));
  calibrate_int_pipes(ctx->stream, scratch, fmul_per_s, blake3_per_s);
  API_END(ctx)
}

int gbz_party_sumcheck_rounds(uint64_t M, int N, int offset) {
  if (!is_pow2(M) || N < 1 || !is_pow2((uint64_t)N) || offset < 0) return -1;
  return party_sumcheck_rounds(M, N, offset, nullptr);
}

gbz_status gbz_party_sumcheck(gbz_ctx *ctx, int form, const uint64_t *v1, const uint64_t *v2, const uint64_t *v3,
                              uint64_t M, int N, const uint64_t *w, int offset, uint64_t *fs_state, gbz_prng *prng,
                              uint64_t *y, uint64_t *polys, uint64_t *challenges, uint64_t *fin, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  if (form != SC_QUADRATIC && form != SC_CUBIC) throw ArgError("party sumcheck: form must be quadratic or cubic");
  const int nv = form_vectors(form), nc = form_coeffs(form);
  need(v1, "v1");
  need(v2, "v2");
  if (form == SC_CUBIC) need(v3, "v3");
  need(fs_state, "fs_state");
  need(prng, "prng");
  need(y, "y");
  need(polys, "polys");
  need(challenges, "challenges");
  need(fin, "fin");
  check_pow2(M, "party sumcheck: M");
  if (N < 1 || N > 4096 || !is_pow2((uint64_t)N)) throw ArgError("party sumcheck: N must be a power of two in [1, 4096]");
  if (offset < 0 || offset > 40) throw ArgError("party sumcheck: offset out of range");
  const uint64_t total = M * (uint64_t)N;
  if (ilog2(total) > kMaxLogN) throw ArgError("party sumcheck: N * M above 2^28");
  const int rounds = party_sumcheck_rounds(M, N, offset, nullptr);
  const fe *src[3] = {(const fe *)v1, (const fe *)v2, (const fe *)v3};
  const fe *dv[3] = {nullptr, nullptr, nullptr};
  for (int k = 0; k < nv; k++) dv[k] = dev_view(ctx, 40 + k, src[k], 16 * total, mem, true);
  fe *dw = nullptr;
  if (form == SC_CUBIC) {
    std::vector<fe> hw(N, fe_one());
    if (w)
      for (int p = 0; p < N; p++) hw[p] = fe_make(w[2 * p], w[2 * p + 1]);
    dw = (fe *)ctx->buf(43, 16 * (uint64_t)N);
    GBZ_CUDA(cudaMemcpyAsync(dw, hw.data(), 16 * (uint64_t)N, cudaMemcpyHostToDevice, ctx->stream));
    GBZ_CUDA(cudaStreamSynchronize(ctx->stream));  // hw is a host temporary
  }
  RoundState hs;
  hs.fs = fe_make(fs_state[0], fs_state[1]);
  std::memcpy(&hs.prng, prng, sizeof(glibc_prng));
  hs.y = fe_make(y[0], y[1]);
  hs.error = 0;
  RoundState *dst = (RoundState *)ctx->buf(44, sizeof(RoundState));
  GBZ_CUDA(cudaMemcpyAsync(dst, &hs, sizeof(hs), cudaMemcpyHostToDevice, ctx->stream));
  fe *scratch[12];
  for (int k = 0; k < 12; k++) scratch[k] = (fe *)ctx->buf(60 + k, 16 * std::max<uint64_t>(total / 2, 1));
  fe *partial = (fe *)ctx->buf(56, 16 * 4 * (uint64_t)round_blocks(std::max<uint64_t>(total / 2, 1)));
  fe *dpolys = (fe *)ctx->buf(45, 16 * (uint64_t)nc * std::max(rounds, 1));
  fe *dchal = (fe *)ctx->buf(46, 16 * (uint64_t)std::max(rounds, 1));
  fe *dfin = (fe *)ctx->buf(47, 16 * 3);
  fe *ddrawn = (fe *)ctx->buf(49, 16 * (uint64_t)std::max(rounds, 1));
  party_sumcheck_enqueue(form, dv, M, N, dw, offset, dst, scratch, partial, dpolys, dchal, dfin, ddrawn,
                         ctx->side_stream(), ctx->stream);
  if (rounds) {
    GBZ_CUDA(cudaMemcpyAsync(polys, dpolys, 16 * (uint64_t)nc * rounds, cudaMemcpyDeviceToHost, ctx->stream));
    GBZ_CUDA(cudaMemcpyAsync(challenges, dchal, 16 * (uint64_t)rounds, cudaMemcpyDeviceToHost, ctx->stream));
  }
  GBZ_CUDA(cudaMemcpyAsync(fin, dfin, 16 * (uint64_t)nv, cudaMemcpyDeviceToHost, ctx->stream));
  GBZ_CUDA(cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream));
  GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
  fs_state[0] = hs.fs.re;
  fs_state[1] = hs.fs.im;
  std::memcpy(prng, &hs.prng, sizeof(glibc_prng));
  y[0] = hs.y.re;
  y[1] = hs.y.im;
  if (hs.error) return fail(ctx, GBZ_ECHECK, "party sumcheck: a round polynomial did not match the running claim");
  API_END(ctx)
}

uint64_t gbz_whir_open_transcript_bytes(int logn, int rate) {
  try {
    ProofPlan p;
    p.logn = logn;
    p.rate = rate;
    if (logn < 3 || logn > 26 || rate < 2 || rate > 64 || !is_pow2((uint64_t)rate)) return 0;
    p.n = 1ull << logn;
    p.L = p.n * (uint64_t)rate;
    OpenOnly o{};
    enqueue_proof(p, nullptr, 1, nullptr, true, false, &o);
    return p.layout.len;
  } catch (...) {
    return 0;
  }
}

gbz_status gbz_whir_open(gbz_ctx *ctx, const uint64_t *arr, int logn, int rate, const uint64_t *codeword,
                         const uint64_t *point, const uint64_t *K, gbz_prng *prng, uint8_t *transcript,
                         uint64_t capacity, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(arr, "arr");
  need(codeword, "codeword");
  need(point, "point");
  need(K, "K");
  need(prng, "prng");
  need(transcript, "transcript");
  const uint64_t bytes = gbz_whir_open_transcript_bytes(logn, rate);
  if (!bytes) throw ArgError("whir open: unsupported shape (3 <= logn, rate a power of two in [2, 64], rate * 2^logn <= 2^26)");
  if (capacity < bytes) return fail(ctx, GBZ_ESMALL, "transcript buffer smaller than gbz_whir_open_transcript_bytes");
  auto key = std::make_pair(logn, rate);
  auto it = ctx->plans.find(key);
  if (it == ctx->plans.end()) it = ctx->plans.emplace(key, plan_create(logn, rate)).first;
  ProofPlan &p = *it->second;
  p.prof = nullptr;
  plan_prepare_open(p);
  if (p.open_transcript_bytes != bytes) throw ArgError("whir open: transcript layout mismatch");
  cudaStream_t s = ctx->stream;
  OpenOnly o{};
  uint64_t Kw[2];
  if (mem == GBZ_MEM_HOST) {
    GBZ_CUDA(cudaMemcpyAsync(p.w, arr, 16 * p.n, cudaMemcpyHostToDevice, s));
    GBZ_CUDA(cudaMemcpyAsync(p.cw[0], codeword, 16 * p.L, cudaMemcpyHostToDevice, s));
    fe *dpt = (fe *)ctx->buf(0, 16ull * logn);
    GBZ_CUDA(cudaMemcpyAsync(dpt, point, 16ull * logn, cudaMemcpyHostToDevice, s));
    o.codeword = p.cw[0];
    o.point = dpt;
    Kw[0] = K[0];
    Kw[1] = K[1];
  } else {
    o.codeword = (const fe *)codeword;
    o.point = (const fe *)point;
    GBZ_CUDA(cudaMemcpyAsync(Kw, K, 16, cudaMemcpyDeviceToHost, s));
    GBZ_CUDA(cudaStreamSynchronize(s));
  }
  o.K = fe_make(Kw[0], Kw[1]);
  static_assert(sizeof(gbz_prng) == sizeof(glibc_prng), "gbz_prng layout");
  std::memcpy(&o.prng, prng, sizeof(glibc_prng));
  const fe *w = mem == GBZ_MEM_HOST ? p.w : (const fe *)arr;
  enqueue_proof(p, w, 0, s, false, false, &o);
  GBZ_CUDA(cudaMemcpyAsync(transcript, p.open_transcript, bytes,
                           mem == GBZ_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
  glibc_prng after;
  GBZ_CUDA(cudaMemcpyAsync(&after, &p.st->prng, sizeof(glibc_prng), cudaMemcpyDeviceToHost, s));
  const uint32_t err = plan_error_flags(p, s);  // synchronises s
  std::memcpy(prng, &after, sizeof(glibc_prng));
  if (err) return fail(ctx, GBZ_ECHECK, "whir open: a round message did not match the running claim");
  API_END(ctx)
}

uint64_t gbz_prove_transcript_bytes(int logn, int rate) {
  try {
    // Layout only: build a throwaway plan-free layout by a dry enqueue.
    ProofPlan p;
    p.logn = logn;
    p.rate = rate;
    if (logn < 3 || logn > 26 || rate < 2 || rate > 64 || !is_pow2((uint64_t)rate)) return 0;
    p.n = 1ull << logn;
    p.L = p.n * (uint64_t)rate;
    enqueue_proof(p, nullptr, 1, nullptr, true);
    return p.layout.len;
  } catch (...) {
    return 0;
  }
}

gbz_status gbz_prove(gbz_ctx *ctx, const uint64_t *witness, int logn, int rate, uint32_t prng_seed,
                     uint8_t *transcript, uint64_t capacity, int mem) {
  API_BEGIN(ctx)
  check_mem(mem);
  need(witness, "witness");
  need(transcript, "transcript");
  auto key = std::make_pair(logn, rate);
  auto it = ctx->plans.find(key);
  if (it == ctx->plans.end()) it = ctx->plans.emplace(key, plan_create(logn, rate)).first;
  ProofPlan &p = *it->second;
  if (ctx->profiling) {
    auto &pr = ctx->profilers[key];
    if (!pr) pr.reset(new Profiler());
    pr->enabled = true;
    p.prof = pr.get();
  } else {
    p.prof = nullptr;
  }
  if (capacity < p.transcript_bytes) return fail(ctx, GBZ_ESMALL, "transcript buffer smaller than gbz_prove_transcript_bytes");
  const fe *w;
  if (mem == GBZ_MEM_HOST) {
    GBZ_CUDA(cudaMemcpyAsync(p.w, witness, 16 * p.n, cudaMemcpyHostToDevice, ctx->stream));
    w = p.w;
  } else {
    w = (const fe *)witness;
  }
  // Replay a captured graph of the proof (fewer launch gaps between the
  // many small protocol kernels); direct launches when profiling or when the
  // stream is a default stream, which cannot be captured.
  const bool capturable = ctx->stream != nullptr && ctx->stream != cudaStreamLegacy &&
                          ctx->stream != cudaStreamPerThread;
  if (!ctx->profiling && ctx->graphs && capturable) launch_proof_graph(p, w, prng_seed, ctx->stream);
  else enqueue_proof(p, w, prng_seed, ctx->stream, false);
  GBZ_CUDA(cudaMemcpyAsync(transcript, p.transcript, p.transcript_bytes,
                           mem == GBZ_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, ctx->stream));
  if (mem == GBZ_MEM_HOST) {
    if (plan_error_flags(p, ctx->stream)) return fail(ctx, GBZ_ECHECK, "a sumcheck round message did not match its claim");
  }
  API_END(ctx)
}

}  // extern "C"
