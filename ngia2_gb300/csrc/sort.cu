// sort.cu -- device primitives: segmented stable LSD radix sort of (u32 key,
// u32 value) pairs and device-wide exclusive scans.  Hand-written; no library
// sort or scan is used.
//
// Radix sort: 8-bit digits, one pass per digit, three kernels per pass:
//   1. histogram: per (segment, tile of 4096) digit counts;
//   2. scan: per segment, exclusive scan of the counts in digit-major order,
//      giving every (digit, tile) its first output slot;
//   3. scatter: each warp of a tile ranks its contiguous sub-tile stably
//      (equal digits within a round found by eight ballots, warp-private
//      running slots per digit) and writes the keys to their slots.
// Stability makes the passes compose into a sort by (key, input order); with
// values = input index that is exactly a sort by (key, index).
#include <mutex>

#include "kernels.cuh"

namespace ngia {

constexpr uint32_t kTile = 4096;
constexpr uint32_t kSortThreads = 256;
constexpr uint32_t kSortWarps = kSortThreads / 32;

__global__ void __launch_bounds__(kSortThreads)
rs_hist_kernel(const uint32_t *__restrict__ keys, uint32_t seg_len, int shift,
               uint32_t ntiles, uint32_t *__restrict__ counts) {
  __shared__ uint32_t h[kSortWarps][256];
  const uint32_t seg = blockIdx.y, tile = blockIdx.x, warp = threadIdx.x >> 5;
  const uint32_t *k = keys + (size_t)seg * seg_len + tile * kTile + threadIdx.x;
  const uint32_t cnt = seg_len - tile * kTile < kTile ? seg_len - tile * kTile : kTile;
  uint32_t v[kTile / kSortThreads];  // every load in flight before the counts
#pragma unroll
  for (uint32_t j = 0; j < kTile / kSortThreads; ++j)
    v[j] = threadIdx.x + j * kSortThreads < cnt ? k[j * kSortThreads] : 0u;
  for (uint32_t d = threadIdx.x; d < kSortWarps * 256; d += kSortThreads) (&h[0][0])[d] = 0;
  __syncthreads();
#pragma unroll
  for (uint32_t j = 0; j < kTile / kSortThreads; ++j)
    if (threadIdx.x + j * kSortThreads < cnt) atomicAdd(&h[warp][(v[j] >> shift) & 255u], 1u);
  __syncthreads();
  uint32_t c = 0;
#pragma unroll
  for (uint32_t w = 0; w < kSortWarps; ++w) c += h[w][threadIdx.x];
  counts[((size_t)seg * 256 + threadIdx.x) * ntiles + tile] = c;
}

// In-place exclusive scan of `len` u32 per segment (one block per segment).
__global__ void __launch_bounds__(1024)
segment_scan_kernel(uint32_t *__restrict__ data, uint32_t len) {
  __shared__ uint32_t part[1024];
  uint32_t *d = data + (size_t)blockIdx.x * len;
  const uint32_t per = (len + 1023) / 1024;
  const uint32_t beg = threadIdx.x * per, end = min(beg + per, len);
  uint32_t s = 0;
  for (uint32_t i = beg; i < end; ++i) s += d[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t off = 1; off < 1024; off <<= 1) {  // Hillis-Steele inclusive
    uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
  for (uint32_t i = beg; i < end; ++i) {
    const uint32_t v = d[i];
    d[i] = run;
    run += v;
  }
}

// Segments longer than one block's share (the digit counts of a big single
// segment) are scanned by many blocks: chunk sums, a scan of the sums per
// segment, then each chunk scanned from its offset.
constexpr uint32_t kScanChunk = 8192;  // u32 per block, 8 per thread

__device__ __forceinline__ uint32_t block_excl_scan_u32(uint32_t v, uint32_t *sh,
                                                        uint32_t &total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < blockDim.x / 32 ? sh[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, w, o);
      if (lane >= (uint32_t)o) w += y;
    }
    sh[lane] = w;
  }
  __syncthreads();
  total = sh[blockDim.x / 32 - 1];
  const uint32_t before = warp ? sh[warp - 1] : 0u;
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(1024)
chunk_sum_kernel(const uint32_t *__restrict__ data, uint32_t len, uint32_t nchunks,
                 uint32_t *__restrict__ sums) {
  __shared__ uint32_t sh[32];
  const uint32_t *d = data + (size_t)blockIdx.y * len;
  const uint32_t beg = blockIdx.x * kScanChunk + threadIdx.x * 8;
  uint32_t v = 0;
#pragma unroll
  for (uint32_t k = 0; k < 8; ++k)
    if (beg + k < len) v += d[beg + k];
  uint32_t total;
  block_excl_scan_u32(v, sh, total);
  if (threadIdx.x == 0) sums[(size_t)blockIdx.y * nchunks + blockIdx.x] = total;
}

// exclusive scan of each segment's chunk sums (one block per segment)
__global__ void __launch_bounds__(1024)
chunk_sums_scan_kernel(uint32_t *__restrict__ sums, uint32_t nchunks) {
  __shared__ uint32_t sh[32];
  uint32_t *d = sums + (size_t)blockIdx.x * nchunks;
  uint32_t run = 0;
  for (uint32_t b = 0; b < nchunks; b += 1024) {  // block-uniform
    const uint32_t i = b + threadIdx.x;
    const uint32_t v = i < nchunks ? d[i] : 0u;
    uint32_t total;
    const uint32_t x = block_excl_scan_u32(v, sh, total);
    if (i < nchunks) d[i] = run + x;
    run += total;
  }
}

__global__ void __launch_bounds__(1024)
chunk_apply_kernel(uint32_t *__restrict__ data, uint32_t len, uint32_t nchunks,
                   const uint32_t *__restrict__ sums) {
  __shared__ uint32_t sh[32];
  uint32_t *d = data + (size_t)blockIdx.y * len;
  const uint32_t beg = blockIdx.x * kScanChunk + threadIdx.x * 8;
  uint32_t v[8], s = 0;
#pragma unroll
  for (uint32_t k = 0; k < 8; ++k) {
    v[k] = beg + k < len ? d[beg + k] : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t run = block_excl_scan_u32(s, sh, total) +
                 sums[(size_t)blockIdx.y * nchunks + blockIdx.x];
#pragma unroll
  for (uint32_t k = 0; k < 8; ++k) {
    if (beg + k < len) d[beg + k] = run;
    run += v[k];
  }
}

// Counts up to kScanOneBlock per segment are scanned by one block per segment
// (16 per thread: one launch instead of three); longer ones in chunks.
constexpr uint32_t kScanOneBlock = 16384;
static uint32_t scan_chunks(uint32_t ntiles) {
  const uint32_t len = 256 * ntiles;
  return len > kScanOneBlock ? ceil_div(len, kScanChunk) : 0u;
}

// Scatter of one tile of kTile keys and values.  Each warp takes a contiguous
// sub-tile of kWarpKeys, its keys held in registers (lane l: keys 32r + l)
// and its values, when the pass has any, copied into shared memory by
// cp.async while the keys are ranked:
//   1. rank: per round of 32 keys, each lane sets its bit in a warp-private
//      mask of its digit (a shared-memory atomic OR, one per run of equal
//      digits in neighbouring lanes), reads the mask back --
//      the lanes sharing its digit -- and takes its slot among them after the
//      warp's running count of that digit, which the lowest of them advances;
//      three mask buffers in rotation, so one warp barrier per round;
//   2. the block turns the warp counts into tile-local slots per (warp, digit)
//      and the scanned offsets into each digit's global first slot;
//   3. keys and values go to their tile-local slots in shared memory (the
//      tile sorted by digit), then out in that order: consecutive threads
//      write consecutive slots of a digit's run, so stores coalesce.
// Stable: warps hold consecutive sub-tiles, rounds and lanes go in key order.
constexpr uint32_t kWarpKeys = kTile / kSortWarps;
constexpr uint32_t kRounds = kWarpKeys / 32;
constexpr uint32_t kMaskBufs = 3;
constexpr uint32_t kMaskWords = kSortWarps * 256;  // one buffer
// shared memory, in u32: the sorted keys, the sorted values (where the values
// are staged until the keys are placed), a spare region, per-warp digit
// counts / slots, per-digit global first slots (less the tile-local one), the
// block scan's warp totals.  Mask buffers 0 and 1 sit in the sorted keys'
// space and buffer 2 in the spare region, clear of the staged values.
constexpr uint32_t kSmKeys = 0;
constexpr uint32_t kSmVals = kTile;
constexpr uint32_t kSmSpare = 2 * kTile;
constexpr uint32_t kSmCount = kSmSpare + kMaskWords;
constexpr uint32_t kSmGlobal = kSmCount + kSortWarps * 256;
constexpr uint32_t kSmWarpSum = kSmGlobal + 256;
constexpr uint32_t kSmWords = kSmWarpSum + kSortWarps;
static_assert(2 * kMaskWords <= kTile, "mask buffers 0 and 1 fit the sorted keys' space");
static_assert(kSortThreads == 256, "one thread per digit in the block scan");

__device__ __forceinline__ void cp_async4(uint32_t *smem, const uint32_t *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem));
}

template <bool kValues>
__global__ void __launch_bounds__(kSortThreads, 4)
rs_scatter_kernel(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                  uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                  uint32_t seg_len, int shift, uint32_t ntiles,
                  const uint32_t *__restrict__ offsets) {
  extern __shared__ uint32_t rs_smem[];
  uint32_t *sk = rs_smem + kSmKeys, *sv = rs_smem + kSmVals;
  uint32_t(*count)[256] = reinterpret_cast<uint32_t(*)[256]>(rs_smem + kSmCount);
  uint32_t *global = rs_smem + kSmGlobal;
  uint32_t *wsum = rs_smem + kSmWarpSum;
  const uint32_t seg = blockIdx.y, tile = blockIdx.x;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const size_t so = (size_t)seg * seg_len;
  const uint32_t t0 = tile * kTile;
  const uint32_t cnt = seg_len - t0 < kTile ? seg_len - t0 : kTile;  // keys in this tile
  const uint32_t w0 = warp * kWarpKeys;                              // the warp's first key
  const size_t my = so + t0 + w0 + lane;  // the lane's first key; round r adds 32r
  const uint32_t mine = cnt > w0 + lane ? cnt - w0 - lane : 0u;  // round r valid: 32r < mine
  uint32_t key[kRounds], rank[kRounds];
#pragma unroll
  for (uint32_t r = 0; r < kRounds; ++r) key[r] = 32 * r < mine ? kin[my + 32 * r] : 0u;
  if constexpr (kValues) {  // the lane's values into the staging space, asynchronously
#pragma unroll
    for (uint32_t r = 0; r < kRounds; ++r)
      if (32 * r < mine) cp_async4(sv + w0 + 32 * r + lane, vin + my + 32 * r);
    asm volatile("cp.async.commit_group;\n" ::);
  }
  {
    uint32_t *m0 = rs_smem + kSmKeys, *m2 = rs_smem + kSmSpare;
    for (uint32_t i = threadIdx.x; i < 2 * kMaskWords; i += kSortThreads) m0[i] = 0;
    for (uint32_t i = threadIdx.x; i < kMaskWords; i += kSortThreads) m2[i] = 0;
  }
#pragma unroll
  for (uint32_t w = 0; w < kSortWarps; ++w) count[w][threadIdx.x] = 0;
  __syncthreads();

  // 1. rank within the warp
  const uint32_t bit = 1u << lane, lt_mask = bit - 1u;
  uint32_t *wcount = count[warp];
  uint32_t *clear = nullptr;  // the entry this lane led last round (cleared one round later)
#pragma unroll
  for (uint32_t r = 0; r < kRounds; ++r) {
    const bool valid = 32 * r < mine;
    const uint32_t d = (key[r] >> shift) & 255u;
    const uint32_t b = r % kMaskBufs;
    uint32_t *m = rs_smem + (b < 2 ? kSmKeys + b * kMaskWords : kSmSpare) + warp * 256;
    // a run of lanes with one digit (sorted input repeats keys) sets its bits
    // with one atomic: same-address atomics of a warp serialise.  Valid lanes
    // are a prefix of the warp.
    const uint32_t dprev = __shfl_up_sync(kFull, d, 1);
    const bool start = valid && (lane == 0 || dprev != d);
    const uint32_t starts = __ballot_sync(kFull, start);
    const uint32_t vmask = __ballot_sync(kFull, valid);
    if (start) {
      const uint32_t above = starts & ~((2u << lane) - 1u);  // later run starts
      const uint32_t end = above ? (uint32_t)__ffs(above) - 1u : 32u;
      const uint32_t upto = end == 32u ? kFull : (1u << end) - 1u;
      atomicOr(m + d, upto & ~lt_mask & vmask);
    }
    __syncwarp();
    const uint32_t peers = valid ? m[d] : 0u;
    const uint32_t leader = peers ? __ffs(peers) - 1u : lane;
    const uint32_t seen = valid && leader == lane ? wcount[d] : 0u;  // the leaders read
    const uint32_t base = __shfl_sync(kFull, seen, leader);
    // last round's masks: every lane has read them (the barrier above)
    if (clear) *clear = 0u;
    clear = nullptr;
    if (valid && (peers & lt_mask) == 0) {
      wcount[d] = base + __popc(peers);
      clear = m + d;
    }
    rank[r] = base + __popc(peers & lt_mask);
  }
  __syncthreads();

  // 2. tile-local slots per (warp, digit) and each digit's global first slot
  {
    const uint32_t t = threadIdx.x;  // digit t
    uint32_t tot = 0;
#pragma unroll
    for (uint32_t w = 0; w < kSortWarps; ++w) {
      const uint32_t c = count[w][t];
      count[w][t] = tot;
      tot += c;
    }
    uint32_t x = tot;  // inclusive scan over digits
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, x, o);
      if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    uint32_t before = 0;
#pragma unroll
    for (uint32_t w = 0; w < kSortWarps; ++w) before += w < warp ? wsum[w] : 0u;
    const uint32_t first = before + x - tot;  // tile-local first slot of digit t
#pragma unroll
    for (uint32_t w = 0; w < kSortWarps; ++w) count[w][t] += first;
    global[t] = offsets[((size_t)seg * 256 + t) * ntiles + tile] - first;
  }
  __syncthreads();

  // 3. the tile sorted by digit in shared memory, then written out in order
#pragma unroll
  for (uint32_t r = 0; r < kRounds; ++r) {
    if (32 * r < mine) {
      rank[r] += wcount[(key[r] >> shift) & 255u];  // now the key's slot
      sk[rank[r]] = key[r];
    }
  }
  if constexpr (kValues) {
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    uint32_t val[kRounds];  // the lane's own staged values, then their slots
#pragma unroll
    for (uint32_t r = 0; r < kRounds; ++r) val[r] = sv[w0 + 32 * r + lane];
    __syncthreads();  // every staged value read before any is overwritten
#pragma unroll
    for (uint32_t r = 0; r < kRounds; ++r)
      if (32 * r < mine) sv[rank[r]] = val[r];
  } else {
#pragma unroll
    for (uint32_t r = 0; r < kRounds; ++r)
      if (32 * r < mine) sv[rank[r]] = t0 + w0 + lane + 32 * r;
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < cnt; i += kSortThreads) {
    const uint32_t k = sk[i];
    const uint32_t pos = global[(k >> shift) & 255u] + i;  // mod 2^32: the digit's slot
    if (pos < seg_len) {
      kout[so + pos] = k;
      vout[so + pos] = sv[i];
    }
  }
}

constexpr size_t kScatterSmem = kSmWords * sizeof(uint32_t);

// Above 48 KB of dynamic shared memory a kernel must opt in, once per device.
static int scatter_smem_opt_in() {
  static std::mutex mu;
  static bool done[128] = {};
  int dev = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return NGIA_ERR_ARG;
  std::lock_guard<std::mutex> lock(mu);
  if (!done[dev]) {
    NGIA_CUDA(cudaFuncSetAttribute(rs_scatter_kernel<false>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kScatterSmem));
    NGIA_CUDA(cudaFuncSetAttribute(rs_scatter_kernel<true>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kScatterSmem));
    done[dev] = true;
  }
  return NGIA_OK;
}

int sort_prepare() { return scatter_smem_opt_in(); }

size_t radix_sort_scratch_bytes(uint32_t seg_len, uint32_t segs) {
  const size_t ntiles = ceil_div<size_t>(seg_len, kTile);
  const size_t n = (size_t)seg_len * segs;
  return 2 * n * sizeof(uint32_t) + segs * 256 * ntiles * sizeof(uint32_t) +
         (size_t)segs * scan_chunks((uint32_t)ntiles) * sizeof(uint32_t) + 256;
}

int radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in,
                     uint32_t *keys_out, uint32_t *vals_out, uint32_t seg_len,
                     uint32_t segs, int begin_bit, int end_bit, void *scratch,
                     cudaStream_t s) {
  if (seg_len == 0 || segs == 0) return NGIA_OK;
  const uint32_t ntiles = ceil_div(seg_len, kTile);
  const size_t n = (size_t)seg_len * segs;
  uint32_t *tk = static_cast<uint32_t *>(scratch);
  uint32_t *tv = tk + n;
  uint32_t *counts = tv + n;
  uint32_t *sums = counts + (size_t)segs * 256 * ntiles;
  const uint32_t nchunks = scan_chunks(ntiles);
  const int passes = (end_bit - begin_bit + 7) / 8;
  if (passes <= 0) {
    NGIA_CUDA(cudaMemcpyAsync(keys_out, keys_in, n * 4, cudaMemcpyDeviceToDevice, s));
    if (vals_in) {
      NGIA_CUDA(cudaMemcpyAsync(vals_out, vals_in, n * 4, cudaMemcpyDeviceToDevice, s));
      return NGIA_OK;
    }
    return NGIA_ERR_ARG;  // identity values with zero passes: caller's job
  }
  NGIA_TRY(scatter_smem_opt_in());
  const uint32_t *sk = keys_in, *sv = vals_in;
  for (int p = 0; p < passes; ++p) {
    // the last pass lands in keys_out / vals_out
    const bool to_out = ((passes - 1 - p) % 2) == 0;
    uint32_t *dk = to_out ? keys_out : tk, *dv = to_out ? vals_out : tv;
    const int shift = begin_bit + 8 * p;
    dim3 grid(ntiles, segs);
    rs_hist_kernel<<<grid, kSortThreads, 0, s>>>(sk, seg_len, shift, ntiles, counts);
    NGIA_LAUNCHED();
    if (nchunks == 0) {
      segment_scan_kernel<<<segs, 1024, 0, s>>>(counts, 256 * ntiles);
      NGIA_LAUNCHED();
    } else {
      chunk_sum_kernel<<<dim3(nchunks, segs), 1024, 0, s>>>(counts, 256 * ntiles, nchunks, sums);
      NGIA_LAUNCHED();
      chunk_sums_scan_kernel<<<segs, 1024, 0, s>>>(sums, nchunks);
      NGIA_LAUNCHED();
      chunk_apply_kernel<<<dim3(nchunks, segs), 1024, 0, s>>>(counts, 256 * ntiles, nchunks,
                                                             sums);
      NGIA_LAUNCHED();
    }
    if (sv)
      rs_scatter_kernel<true><<<grid, kSortThreads, kScatterSmem, s>>>(sk, sv, dk, dv, seg_len,
                                                                       shift, ntiles, counts);
    else
      rs_scatter_kernel<false><<<grid, kSortThreads, kScatterSmem, s>>>(sk, sv, dk, dv, seg_len,
                                                                        shift, ntiles, counts);
    NGIA_LAUNCHED();
    sk = dk;
    sv = dv;
  }
  return NGIA_OK;
}

// ---- device-wide exclusive scan (u32 in, u64 out) ---------------------------------
constexpr uint32_t kScanThreads = 256, kScanItems = 8;
constexpr uint32_t kScanBlock = kScanThreads * kScanItems;

__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, uint64_t *sh,
                                                    uint64_t &total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint64_t w = lane < blockDim.x / 32 ? sh[lane] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t y = __shfl_up_sync(kFull, w, o);
      if (lane >= (uint32_t)o) w += y;
    }
    sh[lane] = w;
  }
  __syncthreads();
  total = sh[blockDim.x / 32 - 1];
  const uint64_t before = warp ? sh[warp - 1] : 0ull;
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads)
scan_reduce_kernel(const uint32_t *__restrict__ in, uint32_t n, uint64_t *__restrict__ sums) {
  __shared__ uint64_t sh[32];
  const size_t beg = (size_t)blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  uint64_t s = 0;
#pragma unroll
  for (uint32_t k = 0; k < kScanItems; ++k)
    if (beg + k < n) s += in[beg + k];
  uint64_t total;
  block_excl_scan(s, sh, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Exclusive scan of the block sums by one block, looping over chunks.
__global__ void __launch_bounds__(kScanThreads)
scan_sums_kernel(uint64_t *__restrict__ sums, uint32_t nb, uint64_t *__restrict__ grand) {
  __shared__ uint64_t sh[32];
  uint64_t carry = 0;
  for (uint32_t c = 0; c < nb; c += kScanThreads) {
    const uint32_t i = c + threadIdx.x;
    const uint64_t v = i < nb ? sums[i] : 0ull;
    uint64_t total;
    const uint64_t ex = block_excl_scan(v, sh, total);
    if (i < nb) sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0 && grand) *grand = carry;
}

__global__ void __launch_bounds__(kScanThreads)
scan_apply_kernel(const uint32_t *__restrict__ in, uint32_t n,
                  const uint64_t *__restrict__ sums, uint64_t *__restrict__ out) {
  __shared__ uint64_t sh[32];
  const size_t beg = (size_t)blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint64_t s = 0;
#pragma unroll
  for (uint32_t k = 0; k < kScanItems; ++k) {
    v[k] = beg + k < n ? in[beg + k] : 0u;
    s += v[k];
  }
  uint64_t total;
  uint64_t run = sums[blockIdx.x] + block_excl_scan(s, sh, total);
#pragma unroll
  for (uint32_t k = 0; k < kScanItems; ++k) {
    if (beg + k < n) out[beg + k] = run;
    run += v[k];
  }
}

size_t scan_scratch_bytes(uint32_t n) {
  return (ceil_div<size_t>(n, kScanBlock) + 1) * sizeof(uint64_t);
}

int exclusive_scan_u64(const uint32_t *in, uint64_t *out, uint32_t n,
                       uint64_t *d_total, void *scratch, cudaStream_t s) {
  if (n == 0) {
    if (d_total) NGIA_CUDA(cudaMemsetAsync(d_total, 0, sizeof(uint64_t), s));
    return NGIA_OK;
  }
  const uint32_t nb = ceil_div(n, kScanBlock);
  uint64_t *sums = static_cast<uint64_t *>(scratch);
  scan_reduce_kernel<<<nb, kScanThreads, 0, s>>>(in, n, sums);
  NGIA_LAUNCHED();
  scan_sums_kernel<<<1, kScanThreads, 0, s>>>(sums, nb, d_total);
  NGIA_LAUNCHED();
  scan_apply_kernel<<<nb, kScanThreads, 0, s>>>(in, n, sums, out);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

}  // namespace ngia
