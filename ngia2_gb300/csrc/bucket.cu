// bucket.cu -- stage (b): band-key bucketing.
//
// Restates MakeDB::groupSignatures (src/makedb.hpp:289-364): for every band,
// sort (signature, index) stably -- the reference's 4-pass LSD radix sort of
// sig<<32|idx -- and link each entry to the previous entry of its signature
// run:  rep[b][idx] = previous idx if the signatures are equal, else idx.
// Equivalently rep[b][i] is the largest j < i with sig[b][j] == sig[b][i].
//
// Device form, per band:
//   1. partition: stable 8-bit radix passes on the signature's low bits, as
//      many as keep the runs of equal low bits (buckets) at about four
//      entries on average -- two passes up to 2^18 sequences, three up to
//      2^26, else all four; each bucket holds its entries in index order;
//   2. resolve (rep_resolve_kernel, rep_resolve_far_kernel): each sorted entry
//      scans back through its bucket to the nearest entry with the same
//      signature, which is its predecessor in index order (none: the entry is
//      its own rep) -- within a tile staged in shared memory for the first
//      steps, one warp per entry 512 entries a step beyond.
// Two or three sort passes instead of four, and the chain written by the
// resolve pass itself.  Equal signatures always share a bucket, so a scan
// only passes entries of other signatures whose low bits collide -- a few on
// average; the loop is bounded by the bucket's start.
#include <mutex>

#include "kernels.cuh"

namespace ngia {

// Partition passes: buckets of n / 2^(8P) <= 4 entries on average.  A build
// may fix the count (1..4; 4 = the full sort, buckets of equal signatures).
#ifndef NGIA_BUCKET_PASSES
#define NGIA_BUCKET_PASSES 0
#endif
static int partition_passes(uint32_t n) {
  if (NGIA_BUCKET_PASSES >= 1 && NGIA_BUCKET_PASSES <= 4) return NGIA_BUCKET_PASSES;
  return n <= (1u << 10) ? 1 : n <= (1u << 18) ? 2 : n <= (1u << 26) ? 3 : 4;
}

// sk, sv: each band's (signature, index) pairs ordered stably by the
// signature's low bits (low_mask).  A block takes tiles of kResolveTile
// sorted entries staged in shared memory (every load in flight at once); each
// entry scans back within its tile for at most kResolveSteps entries.  An
// entry whose scan would go further -- its bucket began before the tile, or
// a long run of another signature with the same low bits lies between it and
// its predecessor -- is listed in `slow` and resolved by
// rep_resolve_far_kernel, one warp per entry and 512 entries per step.  (A
// scan of one thread per entry down to its answer lasted as long as the
// longest one: on the 200k DNA set a few entries scan back over ~2,000
// entries of another signature in global memory, and the kernel took 450 us.)
constexpr uint32_t kResolveTile = 4096;
constexpr uint32_t kResolveThreads = 256;
constexpr uint32_t kResolvePer = kResolveTile / kResolveThreads;
constexpr uint32_t kResolveSteps = 64;

__global__ void __launch_bounds__(kResolveThreads, 7)
rep_resolve_kernel(const uint32_t *__restrict__ sk, const uint32_t *__restrict__ sv,
                   uint32_t n, uint32_t bands, uint32_t low_mask, uint32_t *__restrict__ rep,
                   uint64_t *__restrict__ slow, unsigned int *__restrict__ slow_count) {
  __shared__ uint32_t tk[kResolveTile], tv[kResolveTile];
  const uint64_t total = (uint64_t)n * bands;
  for (uint64_t t0 = (uint64_t)blockIdx.x * kResolveTile; t0 < total;
       t0 += (uint64_t)gridDim.x * kResolveTile) {
    const uint32_t cnt = total - t0 < kResolveTile ? (uint32_t)(total - t0) : kResolveTile;
    {
      uint32_t a[kResolvePer], b[kResolvePer];  // every load in flight, then staged
#pragma unroll
      for (uint32_t j = 0; j < kResolvePer; ++j) {
        const uint32_t k = threadIdx.x + j * kResolveThreads;
        a[j] = k < cnt ? sk[t0 + k] : 0u;
        b[j] = k < cnt ? sv[t0 + k] : 0u;
      }
#pragma unroll
      for (uint32_t j = 0; j < kResolvePer; ++j) {
        const uint32_t k = threadIdx.x + j * kResolveThreads;
        tk[k] = a[j];
        tv[k] = b[j];
      }
    }
    // the tile's bands: the one holding its first entry, and where the next
    // begins (a tile shorter than a band meets at most one boundary)
    const uint64_t band0 = t0 / n;
    const uint64_t next0 = (band0 + 1) * n;
    const bool one_cut = n >= kResolveTile;
    __syncthreads();
#pragma unroll 4
    for (uint32_t j = 0; j < kResolvePer; ++j) {
      const uint32_t k = threadIdx.x + j * kResolveThreads;
      if (k >= cnt) break;
      const uint64_t e = t0 + k;
      const uint64_t first = one_cut ? (e < next0 ? next0 - n : next0) : e / n * n;
      const uint32_t sig = tk[k], self = tv[k], bkt = sig & low_mask;
      // within the tile and the band, at most kResolveSteps entries back
      const uint64_t lo_tile = first > t0 ? first : t0;
      const uint32_t room = (uint32_t)(e - lo_tile);
      const uint32_t reach = room < kResolveSteps ? room : kResolveSteps;
      uint32_t r = self;
      bool settled = false;
      for (uint32_t d = 1; d <= reach; ++d) {
        const uint32_t s = tk[k - d];
        if ((s & low_mask) != bkt) {  // the bucket's start: no predecessor
          settled = true;
          break;
        }
        if (s == sig) {
          r = tv[k - d];
          settled = true;
          break;
        }
      }
      // back at the band's first entry without a match: no predecessor
      if (!settled && reach == room && lo_tile == first) settled = true;
      if (settled) rep[first + self] = r;
      else slow[atomicAdd(slow_count, 1u)] = e;
    }
    __syncthreads();
  }
}

// The listed entries: one warp per entry, lane l testing entries
// base - 1 - 32j - l for j < kFarChunks at each step (all loads in flight
// together, base moving down kFarChunks * 32 a step); the nearest lane holding
// the signature gives the predecessor unless a nearer one is outside the
// bucket (or the band starts first).
constexpr uint32_t kFarChunks = 16;

__global__ void __launch_bounds__(256)
rep_resolve_far_kernel(const uint32_t *__restrict__ sk, const uint32_t *__restrict__ sv,
                       uint32_t n, uint32_t low_mask, const uint64_t *__restrict__ slow,
                       const unsigned int *__restrict__ slow_count, uint32_t *__restrict__ rep) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t count = *slow_count;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < count; w += warps) {
    const uint64_t e = slow[w];
    const uint64_t first = e / n * n;
    const uint32_t sig = sk[e], bkt = sig & low_mask, self = sv[e];
    uint32_t r = self;
    bool done = false;
    for (uint64_t base = e; base > first && !done;) {  // warp-uniform
      uint32_t v[kFarChunks];
      bool in[kFarChunks];
#pragma unroll
      for (uint32_t j = 0; j < kFarChunks; ++j) {
        in[j] = base >= first + 1u + lane + 32u * j;
        v[j] = in[j] ? __ldg(sk + (base - 1u - lane - 32u * j)) : 0u;
      }
#pragma unroll
      for (uint32_t j = 0; j < kFarChunks; ++j) {
        if (done) break;
        const uint32_t hit = __ballot_sync(kFull, in[j] && v[j] == sig);
        const uint32_t out = __ballot_sync(kFull, !in[j] || (v[j] & low_mask) != bkt);
        const uint32_t stop = hit | out;
        if (stop) {
          const uint32_t l = __ffs(stop) - 1u;  // the nearest
          if ((hit >> l) & 1u) r = __ldg(sv + (base - 1u - l - 32u * j));
          done = true;
        }
      }
      base = base >= first + 32u * kFarChunks ? base - 32u * kFarChunks : first;
    }
    if (lane == 0) rep[first + self] = r;
  }
}

size_t bucket_scratch_bytes(uint32_t n, uint32_t bands) {
  return 2 * (size_t)n * bands * sizeof(uint32_t) + radix_sort_scratch_bytes(n, bands);
}

int bucket(const uint32_t *sigs, uint32_t n, uint32_t bands, uint32_t *rep,
           void *scratch, cudaStream_t s) {
  if (n == 0 || bands == 0) return NGIA_OK;
  const size_t total = (size_t)n * bands;
  uint32_t *sk = static_cast<uint32_t *>(scratch);
  uint32_t *sv = sk + total;
  void *sort_scratch = sv + total;
  const int passes = partition_passes(n);
  NGIA_TRY(radix_sort_pairs(sigs, nullptr, sk, sv, n, bands, 0, 8 * passes, sort_scratch, s));
  const uint32_t low_mask = 8 * passes >= 32 ? kFull : (1u << (8 * passes)) - 1u;
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // after the sort its temporary keys hold the list of far entries, and the
  // first word of its digit counts their number
  // (8 * total bytes into the scratch: 8-byte aligned)
  uint64_t *slow = static_cast<uint64_t *>(sort_scratch);
  unsigned int *slow_count = reinterpret_cast<unsigned int *>(slow + total);
  NGIA_CUDA(cudaMemsetAsync(slow_count, 0, sizeof(unsigned int), s));
  // one tile per block (up to 2^31 - 1 blocks), so that the blocks resident
  // on an SM overlap one another's loads, scans and stores
  const size_t want = ceil_div<size_t>(total, kResolveTile);
  const size_t cap = 0x7FFFFFFF;
  rep_resolve_kernel<<<(uint32_t)(want < cap ? want : cap), kResolveThreads, 0, s>>>(
      sk, sv, n, bands, low_mask, rep, slow, slow_count);
  NGIA_LAUNCHED();
  rep_resolve_far_kernel<<<sms * 4, 256, 0, s>>>(sk, sv, n, low_mask, slow, slow_count, rep);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

}  // namespace ngia

extern "C" int ngia_bucket(const uint32_t *d_sigs, uint32_t n, uint32_t bands,
                           uint32_t *d_rep, void *stream) {
  if (bands < 1 || bands > NGIA_BANDS) return NGIA_ERR_ARG;
  if (n == 0) return NGIA_OK;
  if (!d_sigs || !d_rep) return NGIA_ERR_ARG;
  cudaStream_t s = ngia::as_stream(stream);
  void *scratch = nullptr;
  const size_t bytes = ngia::bucket_scratch_bytes(n, bands);
  cudaError_t e = cudaMallocAsync(&scratch, bytes, s);
  if (e != cudaSuccess) {
    ngia::cuda_fail(e);
    return NGIA_ERR_NOMEM;
  }
  int st = ngia::bucket(d_sigs, n, bands, d_rep, scratch, s);
  e = cudaFreeAsync(scratch, s);
  if (st == NGIA_OK && e != cudaSuccess) st = ngia::cuda_fail(e);
  return st;
}

// ---- allocation-free variant ----------------------------------------------------
// Some callers cannot allocate device memory at call time: a plugin living in
// a host application that reserves the whole device up front, a real-time loop
// that must not take the synchronising allocator path, or a memory-capped
// service that forbids allocations once it is serving.  ngia_bucket_noalloc
// gives them the bucketing stage with its scratch in a fixed array that every
// GPU loading this library holds until the process exits.

namespace ngia {

// Largest n * bands the fixed scratch serves (e.g. 16,384 sequences x 64 bands).
constexpr uint64_t kNoAllocMaxElems = 1ull << 20;
// bucket_scratch_bytes(n, bands) for n * bands <= kNoAllocMaxElems and
// bands <= 64: 16 bytes per element plus the per-tile digit counts
// (256 words per tile, at most kNoAllocMaxElems / 4096 + 64 tiles) plus slack.
constexpr size_t kNoAllocScratchBytes =
    16 * kNoAllocMaxElems + 1024 * (kNoAllocMaxElems / 4096 + kBands) + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Host code may not pass g_noalloc_scratch itself to a kernel (on the host it
// names a host-side stand-in); the device address is looked up once per
// device with that device current, and cached.
static void *g_noalloc_ptr[128] = {};
static std::mutex g_noalloc_mutex;

static int noalloc_scratch(void **out, int *dev_out) {
  int dev = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return NGIA_ERR_ARG;
  *dev_out = dev;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    NGIA_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return NGIA_OK;
}

}  // namespace ngia

extern "C" int ngia_bucket_noalloc(const uint32_t *d_sigs, uint32_t n, uint32_t bands,
                                   uint32_t *d_rep, void *stream) {
  using namespace ngia;
  if (bands < 1 || bands > NGIA_BANDS) return NGIA_ERR_ARG;
  if (n == 0) return NGIA_OK;
  if (!d_sigs || !d_rep) return NGIA_ERR_ARG;
  if ((uint64_t)n * bands > kNoAllocMaxElems) return NGIA_ERR_ARG;
  if (bucket_scratch_bytes(n, bands) > kNoAllocScratchBytes) return NGIA_ERR_ARG;
  void *scratch = nullptr;
  int dev = 0;
  NGIA_TRY(noalloc_scratch(&scratch, &dev));
  const int st = bucket(d_sigs, n, bands, d_rep, scratch, as_stream(stream));
  if (st == NGIA_ERR_CUDA) {
    // a failed launch may follow a reset of the device's context, which reloads
    // the module and can move the array: look its address up again next time
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    g_noalloc_ptr[dev] = nullptr;
  }
  return st;
}
