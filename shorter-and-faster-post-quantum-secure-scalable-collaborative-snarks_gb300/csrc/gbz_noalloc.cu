// gbz_whir_update_betas_noalloc: the WHIR beta update without any device
// allocation.
//
// Some callers cannot let the library allocate device memory at call time:
// a proving service that admits requests by free HBM and has already handed
// every byte to request slots, or a host runtime reaching this library
// through a foreign-function boundary under a fixed device-memory budget.
// For them this entry point keeps its working memory in one file-scope
// device array, sized for the largest query count the prover uses, which
// every GPU that loads the library holds until the process exits.
#include <mutex>

#include "../../include/gbz.h"
#include "gbz_internal.cuh"

namespace gbz {
namespace {

// Working memory of one call: the combination weights and roots of the
// queries (a ProofState, of which only q, comb and omega_q are used) and the
// per-query power tables of the direct update kernel.
struct NoAllocScratch {
  ProofState st;
  fe pw[kUpdateBetasScratch];
};

// Maximum: kMaxQueries (256) queries; about 1 MiB.
static __device__ __align__(256) uint8_t g_noalloc_scratch[sizeof(NoAllocScratch)];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array in the current device's context.  The
// host-side symbol is only a stand-in; the address comes from
// cudaGetSymbolAddress with that device current.  Outside a stream capture
// it is looked up on every call (a context created after a device reset, or
// another context made current on the device, has its own copy of the
// array); during a capture the address the last uncaptured call cached for
// the device is used, so that the capture contains no lookup.
cudaError_t scratch_on_current_device(cudaStream_t s, NoAllocScratch **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(s, &cap);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  } else if (!g_scratch_addr[dev]) {
    return cudaErrorStreamCaptureUnsupported;  // no uncaptured call on this device yet
  }
  *out = reinterpret_cast<NoAllocScratch *>(g_scratch_addr[dev]);
  return cudaSuccess;
}

// comb_i = r^(i+1) (also written to `challenges` when given), the query
// reduced mod N, and omega_N^{q_i}.
__global__ void noalloc_prep_kernel(ProofState *st, const int32_t *q, int l, int logN, fe r, fe *challenges) {
  if (threadIdx.x == 0) {
    fe c = r;
    for (int i = 0; i < l; i++) {
      st->comb[i] = c;
      if (challenges) challenges[i] = c;
      c = fmul(c, r);
    }
  }
  const fe om = root_of_unity(logN);
  const uint32_t mask = (1u << logN) - 1;
  for (int i = threadIdx.x; i < l; i += blockDim.x) {
    const uint32_t qr = (uint32_t)q[i] & mask;
    st->q[i] = (int32_t)qr;
    st->omega_q[i] = fpow(om, (uint64_t)qr);
  }
}

}  // namespace
}  // namespace gbz

extern "C" gbz_status gbz_whir_update_betas_noalloc(uint64_t *b, uint64_t nb, const int32_t *queries, int l,
                                                    uint64_t N, const uint64_t *r, uint64_t *challenges,
                                                    void *cuda_stream) {
  using namespace gbz;
  if (!b || !r || (l > 0 && !queries)) return GBZ_EINVAL;
  if (l < 0 || l > kMaxQueries) return GBZ_EINVAL;  // scratch holds at most 256 queries
  if (!is_pow2(N) || ilog2(N) > kMaxLogN) return GBZ_EINVAL;
  if (l == 0) return GBZ_OK;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  NoAllocScratch *scratch = nullptr;
  if (scratch_on_current_device(s, &scratch) != cudaSuccess) return GBZ_ECUDA;
  noalloc_prep_kernel<<<1, 256, 0, s>>>(&scratch->st, queries, l, ilog2(N), fe_make(r[0], r[1]),
                                        reinterpret_cast<fe *>(challenges));
  if (cudaGetLastError() != cudaSuccess) return GBZ_ECUDA;
  if (nb == 0) return GBZ_OK;  // the weights are written; there is nothing to update
  try {
    update_betas_launch(reinterpret_cast<fe *>(b), nb, &scratch->st, l, scratch->pw, s);
  } catch (const CudaError &) {
    return GBZ_ECUDA;
  } catch (const ArgError &) {
    return GBZ_EINVAL;
  }
  return GBZ_OK;
}
