// The library context (gbz_ctx of include/gbz.h) and the helpers every
// translation unit with extern "C" entry points uses: device guard, error
// mapping, argument checks and host/device views of caller buffers.
#pragma once
#include <algorithm>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gbz.h"
#include "gbz_prover.cuh"
#include "gbz_rounds.cuh"
#include "gbz_sched.cuh"

using namespace gbz;

struct gbz_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string last_error;
  std::map<int, std::pair<void *, uint64_t>> scratch;
  // Scratch of calls that make the same sequence of allocations for the
  // same shape (the N-party openings): keyed by the shape, buffer k of a
  // pool serves the call's k-th allocation.
  std::map<std::string, std::vector<std::pair<void *, uint64_t>>> pools;
  std::map<int, NttTables> ntt;
  std::map<std::pair<int, int>, std::unique_ptr<ProofPlan>> plans;
  ProofState *st = nullptr;
  fe *ub_scratch = nullptr;
  bool profiling = false;
  std::map<std::pair<int, int>, std::unique_ptr<Profiler>> profilers;
  std::unique_ptr<Scheduler> sched;
  bool graphs = true;  // gbz_prove replays captured graphs (gbz_set_graphs)
  bool group = true;   // gbz_prove_batch: proofs of one shape share launches (gbz_sched_set_grouping)
  SideStream side;     // second stream of the party sumcheck (created on first use)

  const SideStream &side_stream() {
    if (!side.stream) {
      GBZ_CUDA(cudaStreamCreateWithFlags(&side.stream, cudaStreamNonBlocking));
      GBZ_CUDA(cudaEventCreateWithFlags(&side.fork, cudaEventDisableTiming));
      GBZ_CUDA(cudaEventCreateWithFlags(&side.join, cudaEventDisableTiming));
    }
    return side;
  }

  void *buf(int slot, uint64_t bytes) {
    auto &e = scratch[slot];
    if (e.second < bytes) {
      if (e.first) GBZ_CUDA(cudaFree(e.first));
      e.first = nullptr;
      e.second = 0;
      GBZ_CUDA(cudaMalloc(&e.first, bytes ? bytes : 16));
      e.second = bytes;
    }
    return e.first;
  }
  NttTables &tables(int lg) {
    auto it = ntt.find(lg);
    if (it != ntt.end()) return it->second;
    NttTables t;
    ntt_tables_build(t, lg);
    return ntt.emplace(lg, t).first->second;
  }
};

namespace gbz_api {

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) GBZ_CUDA(cudaSetDevice(dev));
  }
  ~DeviceGuard() {
    int cur;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

// Device buffers of one call: allocated per call and freed at its end, or,
// with a pool, the pool's k-th buffer for the call's k-th allocation (a
// larger or new one replaces it when it is too small).
struct OpenBufs {
  std::vector<void *> owned;
  std::vector<std::pair<void *, uint64_t>> *pool = nullptr;
  size_t next = 0;
  ~OpenBufs() {
    for (void *p : owned) cudaFree(p);
  }
  template <typename T>
  T *alloc(uint64_t count) {
    const uint64_t bytes = std::max<uint64_t>(count * sizeof(T), 16);
    if (pool) {
      auto &P = *pool;
      if (next < P.size() && P[next].second >= bytes) return (T *)P[next++].first;
      void *p = nullptr;
      GBZ_CUDA(cudaMalloc(&p, bytes));
      if (next < P.size()) {
        cudaFree(P[next].first);
        P[next] = {p, bytes};
      } else {
        P.push_back({p, bytes});
      }
      next++;
      return (T *)p;
    }
    void *p = nullptr;
    GBZ_CUDA(cudaMalloc(&p, bytes));
    owned.push_back(p);
    return (T *)p;
  }
};

inline gbz_status fail(gbz_ctx *ctx, gbz_status code, const std::string &msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

#define API_BEGIN(ctx)                                    \
  if (!(ctx)) return GBZ_EINVAL;                          \
  try {                                                   \
    DeviceGuard guard_((ctx)->device);
#define API_END(ctx)                                                                    \
  }                                                                                     \
  catch (const ArgError &e) {                                                           \
    return fail(ctx, GBZ_EINVAL, e.what);                                               \
  }                                                                                     \
  catch (const CudaError &e) {                                                          \
    return fail(ctx, e.err == cudaErrorMemoryAllocation ? GBZ_ENOMEM : GBZ_ECUDA, e.what); \
  }                                                                                     \
  catch (const std::bad_alloc &) {                                                      \
    return fail(ctx, GBZ_ENOMEM, "host allocation failed");                              \
  }                                                                                     \
  return GBZ_OK;

inline void check_mem(int mem) {
  if (mem != GBZ_MEM_HOST && mem != GBZ_MEM_DEVICE) throw ArgError("mem must be GBZ_MEM_HOST or GBZ_MEM_DEVICE");
}
inline void need(const void *p, const char *what) {
  if (!p) throw ArgError(std::string("null pointer: ") + what);
}
inline void check_pow2(uint64_t n, const char *what) {
  if (!is_pow2(n)) throw ArgError(std::string(what) + " must be a power of two");
}

// Device view of a caller buffer: the pointer itself (device memory) or a
// scratch copy (host memory), copied in when `in`.
template <typename T>
T *dev_view(gbz_ctx *ctx, int slot, T *p, uint64_t bytes, int mem, bool in) {
  if (mem == GBZ_MEM_DEVICE) return p;
  T *d = (T *)ctx->buf(slot, bytes);
  if (in && bytes) GBZ_CUDA(cudaMemcpyAsync((void *)d, (const void *)p, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return d;
}
template <typename T>
void copy_out(gbz_ctx *ctx, T *host, const T *dev, uint64_t bytes, int mem) {
  if (mem == GBZ_MEM_DEVICE || !bytes) return;
  GBZ_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
}
inline void finish(gbz_ctx *ctx, int mem) {
  if (mem == GBZ_MEM_HOST) GBZ_CUDA(cudaStreamSynchronize(ctx->stream));
}

// coPCS Encode (coPCS.cpp:131-147) of nrows rows of 2^logrow entries
// (device) into codewords of rate * 2^logrow entries (device), on the
// context's stream; scratch slot 2 holds the intermediate.
void encode_rows_device(gbz_ctx *ctx, const fe *drows, int nrows, int logrow, int rate, int log_rate_offset,
                        fe *dout);

}  // namespace gbz_api
