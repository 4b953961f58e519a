/*
 * cuda_stub.h -- lets the reference's CUDA headers compile as a plain
 * host (OpenMP) program.  TEST INFRASTRUCTURE ONLY: used by ref_build.sh to
 * build the reference's own alignment / Leiden / save code as the CPU oracle
 * and CPU baseline.  Original work; contains no reference code.
 *
 * The alignment kernel becomes an ordinary function called once per job
 * index from an OpenMP loop (SHIM_LAUNCH); the thread index it computes from
 * blockDim/blockIdx/threadIdx comes from a thread-local set by that loop.
 * Managed allocations become malloc; the other runtime calls succeed and do
 * nothing.
 */
#ifndef NGIA_CUDA_STUB_H
#define NGIA_CUDA_STUB_H

#include <cstdint>
#include <cstdlib>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __launch_bounds__(a, b)

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum { cudaFuncCachePreferL1 = 2 };

struct cudaDeviceProp {
  char name[256];
};

static inline const char *cudaGetErrorString(cudaError_t e) {
  return e == cudaSuccess ? "no error" : "host shim error";
}
static inline cudaError_t cudaGetLastError() { return cudaSuccess; }
static inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
static inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
static inline cudaError_t cudaDeviceSetCacheConfig(int) { return cudaSuccess; }
static inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp *p, int) {
  std::strcpy(p->name, "host (OpenMP shim)");
  return cudaSuccess;
}
template <typename T>
static inline cudaError_t cudaMallocManaged(T **p, size_t bytes) {
  *p = static_cast<T *>(std::malloc(bytes ? bytes : 1));
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
static inline cudaError_t cudaFree(void *p) {
  std::free(p);
  return cudaSuccess;
}

static inline int __popc(uint32_t x) { return __builtin_popcount(x); }
static inline int32_t max(int32_t a, int32_t b) { return a > b ? a : b; }
static inline int32_t min(int32_t a, int32_t b) { return a < b ? a : b; }

struct shim_dim3 {
  unsigned x;
};
static thread_local unsigned shim_job_index;
#define blockDim (shim_dim3{1u})
#define blockIdx (shim_dim3{shim_job_index})
#define threadIdx (shim_dim3{0u})

/* One call of the kernel per job index, spread over the OpenMP team. */
#define SHIM_LAUNCH(count, kernel, ...)                              \
  do {                                                               \
    const long shim_n_ = (long)(count);                              \
    _Pragma("omp parallel for schedule(dynamic, 64)")                \
    for (long shim_i_ = 0; shim_i_ < shim_n_; shim_i_++) {           \
      shim_job_index = (unsigned)shim_i_;                            \
      kernel(__VA_ARGS__);                                           \
    }                                                                \
  } while (0)

#endif
