// Integer-pipe calibration: the device's throughput of the two operations
// the ALU-bound kernels are built from, the F_{p^2} multiply (NTT, RS
// folds, coSumcheck block transforms) and the 64-byte Blake3 compression
// (Merkle levels).  These are the denominators of the integer roofline that
// bench.py reports beside the HBM one.
#include "gbz_internal.cuh"

namespace gbz {

namespace {

constexpr int kCalThreads = 256;
constexpr int kChains = 4;

// kChains independent multiply chains per thread (enough independent work
// to keep the pipes busy); the result is stored so nothing is removed.
__global__ void __launch_bounds__(kCalThreads) fmul_peak_kernel(fe *out, int iters, fe seed) {
  const uint32_t t = blockIdx.x * kCalThreads + threadIdx.x;
  fe a[kChains];
  const fe w = fe_make((seed.re + t) & P, (seed.im ^ (t * 0x9E37u)) & P);
#pragma unroll
  for (int k = 0; k < kChains; k++) a[k] = fe_make((seed.re * (k + 3) + t) % P, (seed.im + 77 * k + t) % P);
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < kChains; k++) a[k] = fmul(a[k], w);
  fe s = a[0];
#pragma unroll
  for (int k = 1; k < kChains; k++) s = fadd(s, a[k]);
  out[t] = s;
}

// One chain of compressions per thread: h <- blake3(h || h).
__global__ void __launch_bounds__(kCalThreads) blake3_peak_kernel(uint32_t *out, int iters, uint32_t seed) {
  const uint32_t t = blockIdx.x * kCalThreads + threadIdx.x;
  uint32_t m[16], h[8];
#pragma unroll
  for (int k = 0; k < 8; k++) h[k] = seed * (k + 1) + t;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      m[k] = h[k];
      m[8 + k] = h[k];
    }
    blake3_block64(m, h);
  }
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s ^= h[k];
  out[t] = s;
}

template <typename Launch>
double time_ms(cudaStream_t s, Launch launch) {
  cudaEvent_t a, b;
  GBZ_CUDA(cudaEventCreate(&a));
  GBZ_CUDA(cudaEventCreate(&b));
  launch();  // warm-up
  GBZ_CUDA(cudaEventRecord(a, s));
  launch();
  GBZ_CUDA(cudaEventRecord(b, s));
  GBZ_CUDA(cudaEventSynchronize(b));
  float ms = 0;
  GBZ_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

}  // namespace

void calibrate_int_pipes(cudaStream_t s, void *scratch, double *fmul_per_s, double *blake3_per_s) {
  int dev = 0, sms = 0;
  GBZ_CUDA(cudaGetDevice(&dev));
  GBZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const unsigned blocks = (unsigned)sms * 8;
  const uint64_t threads = (uint64_t)blocks * kCalThreads;
  if (fmul_per_s) {
    const int iters = 2048;
    const double ms = time_ms(s, [&] {
      fmul_peak_kernel<<<blocks, kCalThreads, 0, s>>>((fe *)scratch, iters, fe_make(12345, 678910));
      GBZ_CUDA(cudaGetLastError());
    });
    *fmul_per_s = (double)threads * kChains * iters / (ms * 1e-3);
  }
  if (blake3_per_s) {
    const int iters = 512;
    const double ms = time_ms(s, [&] {
      blake3_peak_kernel<<<blocks, kCalThreads, 0, s>>>((uint32_t *)scratch, iters, 0x5EEDu);
      GBZ_CUDA(cudaGetLastError());
    });
    *blake3_per_s = (double)threads * iters / (ms * 1e-3);
  }
}

uint64_t calibrate_scratch_bytes(int sms) { return (uint64_t)sms * 8 * kCalThreads * sizeof(fe); }

}  // namespace gbz
