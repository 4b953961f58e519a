// probe.cu -- measured integer-ALU ceiling for the roofline of the
// integer-bound kernels (alignment, sketch).
//
// Every thread runs 8 independent chains of lop3.b32 (a three-input logic op,
// the most frequent instruction of the alignment kernels); the chains are
// independent so the measurement is throughput- not latency-bound.  The grid
// covers every SM with 8 blocks of 256 threads.  Result: 32-bit logic
// operations per second, lanes counted individually.
#include "kernels.cuh"

namespace ngia {

constexpr int kProbeChains = 8;
constexpr int kProbeIters = 4096;

__global__ void __launch_bounds__(256) int_peak_kernel(uint32_t seed, uint32_t *sink) {
  uint32_t x[kProbeChains];
#pragma unroll
  for (int c = 0; c < kProbeChains; ++c) x[c] = seed * (threadIdx.x + 1) + c;
  const uint32_t y = seed ^ blockIdx.x, z = ~seed;
  for (int it = 0; it < kProbeIters; ++it) {
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c)
      asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(x[c]) : "r"(y), "r"(z));
  }
  uint32_t r = 0;
#pragma unroll
  for (int c = 0; c < kProbeChains; ++c) r ^= x[c];
  if (r == 0x12345678u) sink[0] = r;  // keeps the chains alive
}

}  // namespace ngia

extern "C" int ngia_int32_peak(void *stream, double *ops_per_s) {
  using namespace ngia;
  if (!ops_per_s) return NGIA_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  uint32_t *sink = nullptr;
  NGIA_CUDA(cudaMallocAsync(&sink, 4, s));
  cudaEvent_t a, b;
  NGIA_CUDA(cudaEventCreate(&a));
  NGIA_CUDA(cudaEventCreate(&b));
  const uint32_t blocks = (uint32_t)sms * 8;
  int_peak_kernel<<<blocks, 256, 0, s>>>(7u, sink);  // warm-up
  NGIA_LAUNCHED();
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    NGIA_CUDA(cudaEventRecord(a, s));
    int_peak_kernel<<<blocks, 256, 0, s>>>(11u + rep, sink);
    NGIA_LAUNCHED();
    NGIA_CUDA(cudaEventRecord(b, s));
    NGIA_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    NGIA_CUDA(cudaEventElapsedTime(&ms, a, b));
    if (ms < best) best = ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  NGIA_CUDA(cudaFreeAsync(sink, s));
  const double ops = (double)blocks * 256.0 * kProbeIters * kProbeChains;
  *ops_per_s = ops / (best * 1e-3);
  return NGIA_OK;
}
