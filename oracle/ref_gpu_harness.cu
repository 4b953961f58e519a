/*
 * ref_gpu_harness.cu -- runs the reference's own alignment kernel
 * (BuildGraph::kernel_dynamic, src/buildGraph.hpp:192-253), built unmodified
 * by nvcc, on a job list read from files.  TEST INFRASTRUCTURE ONLY: the GPU
 * parity tests use it to compare the product kernel with the reference kernel
 * on the same GPU, pair by pair.  Original work; it includes the reference
 * header, it does not reproduce it.
 *
 * usage: ref_gpu_align <packed.u32> <offsets.u64> <jobs.u32> <identity> <out.u32> [groups]
 *   packed.u32  : the packed-record region as little-endian u32 words
 *   offsets.u64 : word offset of each record in that region
 *   jobs.u32    : (rep, tar, 0) u32 triples
 *   out.u32     : the jobs array after the kernel (scores in every third word)
 *   groups      : launches, one per consecutive group of count / groups jobs
 *                 with a device synchronisation after each, as the reference
 *                 launches one kernel per band (default 1)
 * Prints {"count": N, "groups": G, "kernel_ms": T}: T spans every launch.
 */
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "makedb.hpp"
#include "buildGraph.hpp"

static std::vector<char> slurp(const char *path) {
  std::vector<char> b;
  FILE *f = std::fopen(path, "rb");
  if (!f) return b;
  std::fseek(f, 0, SEEK_END);
  long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  b.resize((size_t)n);
  if (n > 0 && std::fread(b.data(), 1, (size_t)n, f) != (size_t)n) b.clear();
  std::fclose(f);
  return b;
}

int main(int argc, char **argv) {
  if (argc != 6 && argc != 7) {
    std::fprintf(stderr, "usage: %s packed offsets jobs identity out [groups]\n", argv[0]);
    return 2;
  }
  const int groups_arg = argc == 7 ? std::atoi(argv[6]) : 1;
  const uint32_t groups = groups_arg > 0 ? (uint32_t)groups_arg : 1u;
  std::vector<char> packed = slurp(argv[1]), offs = slurp(argv[2]),
                    jobs = slurp(argv[3]);
  const unsigned identity = (unsigned)std::atoi(argv[4]);
  const uint32_t count = (uint32_t)(jobs.size() / 12);
  if (packed.empty() || offs.empty()) return 3;
  uint32_t *d_reads = nullptr, *d_jobs = nullptr;
  size_t *d_offs = nullptr;
  if (cudaMalloc(&d_reads, packed.size()) != cudaSuccess) return 4;
  if (cudaMalloc(&d_offs, offs.size()) != cudaSuccess) return 4;
  if (cudaMalloc(&d_jobs, jobs.size() ? jobs.size() : 4) != cudaSuccess) return 4;
  cudaMemcpy(d_reads, packed.data(), packed.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(d_offs, offs.data(), offs.size(), cudaMemcpyHostToDevice);
  if (count) cudaMemcpy(d_jobs, jobs.data(), jobs.size(), cudaMemcpyHostToDevice);
  const float threshold = identity / 100.0f;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a);
  cudaError_t err = cudaSuccess;
  for (uint32_t g = 0; g < groups && err == cudaSuccess; ++g) {
    const uint32_t lo = (uint32_t)((uint64_t)count * g / groups);
    const uint32_t hi = (uint32_t)((uint64_t)count * (g + 1) / groups);
    if (hi > lo)
      BuildGraph::kernel_dynamic<<<(hi - lo + 63) / 64, 64>>>(d_reads, d_offs, d_jobs + 3ull * lo,
                                                              hi - lo, threshold);
    err = cudaDeviceSynchronize();
  }
  cudaEventRecord(b);
  if (err == cudaSuccess) err = cudaDeviceSynchronize();
  if (err == cudaSuccess) err = cudaGetLastError();
  if (err != cudaSuccess) {
    std::fprintf(stderr, "kernel failed: %s\n", cudaGetErrorString(err));
    return 5;
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  if (count) cudaMemcpy(jobs.data(), d_jobs, jobs.size(), cudaMemcpyDeviceToHost);
  FILE *f = std::fopen(argv[5], "wb");
  if (!f) return 6;
  if (count) std::fwrite(jobs.data(), 1, jobs.size(), f);
  std::fclose(f);
  std::printf("{\"count\": %u, \"groups\": %u, \"kernel_ms\": %.6f}\n", count, groups, ms);
  cudaFree(d_reads);
  cudaFree(d_offs);
  cudaFree(d_jobs);
  return 0;
}
