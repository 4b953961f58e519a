// pairs.cu -- candidate collection, width-class binning and edge emission.
//
// Candidates (src/buildGraph.hpp:262-300): target i of band b is a job with
// rep r = rep[b][i] when r != i and len[i] >= len[r] * t.  The reference
// aligns every band's jobs separately, so a pair found in k bands is aligned k
// times and the duplicate edges are removed after sorting
// (src/buildGraph.hpp:357-358).  The score of a pair does not depend on the
// band, so here the candidates of all bands are deduplicated per target
// before alignment: each distinct (rep, tar) pair is aligned once, and the
// emitted edge set is the reference's sorted unique edge list.
//
// Layout: a block loads the rep rows of 32 consecutive targets for all bands
// (coalesced along i), then each warp takes one target: lane l holds bands l
// and l+32; equal reps are found with match_any, and the first band of every
// distinct rep keeps it.  Pairs come out grouped by target in index order.
#include "align.cuh"
#include "kernels.cuh"

namespace ngia {

constexpr uint32_t kTargetsPerBlock = 32;
constexpr uint32_t kPairThreads = 256;

struct TargetScan {
  uint32_t first0, first1;  // ballots of first occurrences (slot 0 / slot 1)
  uint32_t cand;            // candidates including duplicates
  uint32_t v0, v1;
};

__device__ __forceinline__ TargetScan scan_target(const uint32_t *tile_rep /*[64][32]*/,
                                                  uint32_t col, uint32_t i,
                                                  const uint32_t *__restrict__ lens,
                                                  uint32_t bands, float t,
                                                  uint32_t *warp_vals) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const float li = __uint2float_rn(__ldg(lens + i));
  TargetScan ts;
  ts.v0 = lane < bands ? tile_rep[lane * kTargetsPerBlock + col] : i;
  ts.v1 = lane + 32 < bands ? tile_rep[(lane + 32) * kTargetsPerBlock + col] : i;
  const bool ok0 = ts.v0 != i && li >= __fmul_rn(__uint2float_rn(__ldg(lens + ts.v0)), t);
  const bool ok1 = ts.v1 != i && li >= __fmul_rn(__uint2float_rn(__ldg(lens + ts.v1)), t);
  const uint32_t b0 = __ballot_sync(kFull, ok0), b1 = __ballot_sync(kFull, ok1);
  ts.cand = __popc(b0) + __popc(b1);
  const uint32_t tag0 = ok0 ? ts.v0 : (0x80000000u | lane);
  const uint32_t p0 = __match_any_sync(kFull, tag0);
  const bool f0 = ok0 && (p0 & lt_mask) == 0;
  bool f1 = false;
  if (b1) {
    const uint32_t tag1 = ok1 ? ts.v1 : (0xC0000000u | lane);
    const uint32_t p1 = __match_any_sync(kFull, tag1);
    f1 = ok1 && (p1 & lt_mask) == 0;
    warp_vals[lane] = tag0;
    __syncwarp();
    if (f1) {
      for (uint32_t l = 0; l < 32; ++l)
        if (warp_vals[l] == ts.v1) f1 = false;
    }
    __syncwarp();
  }
  ts.first0 = __ballot_sync(kFull, f0);
  ts.first1 = __ballot_sync(kFull, f1);
  return ts;
}

// mode 0: count unique pairs per target; mode 1: write them at offsets[i].
template <int MODE>
__global__ void __launch_bounds__(kPairThreads)
collect_kernel(const uint32_t *__restrict__ rep, const uint32_t *__restrict__ lens,
               uint32_t n, uint32_t bands, float t, uint32_t *__restrict__ ucount,
               unsigned long long *__restrict__ cand_total,
               const uint64_t *__restrict__ offsets, uint2 *__restrict__ pairs) {
  __shared__ uint32_t tile[kBands * kTargetsPerBlock];
  __shared__ uint32_t vals[kPairThreads / 32][32];
  const uint32_t i0 = blockIdx.x * kTargetsPerBlock;
  for (uint32_t e = threadIdx.x; e < bands * kTargetsPerBlock; e += kPairThreads) {
    const uint32_t b = e / kTargetsPerBlock, c = e % kTargetsPerBlock;
    tile[e] = (i0 + c < n) ? rep[(size_t)b * n + i0 + c] : 0u;
  }
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  uint32_t cand_sum = 0;
  for (uint32_t c = warp; c < kTargetsPerBlock; c += kPairThreads / 32) {
    const uint32_t i = i0 + c;
    if (i >= n) break;
    const TargetScan ts = scan_target(tile, c, i, lens, bands, t, vals[warp]);
    cand_sum += ts.cand;
    if (MODE == 0) {
      if (lane == 0) ucount[i] = __popc(ts.first0) + __popc(ts.first1);
    } else {
      const uint32_t lt_mask = (1u << lane) - 1u;
      const uint64_t base = offsets[i];
      if (ts.first0 >> lane & 1u)
        pairs[base + __popc(ts.first0 & lt_mask)] = make_uint2(ts.v0, i);
      if (ts.first1 >> lane & 1u)
        pairs[base + __popc(ts.first0) + __popc(ts.first1 & lt_mask)] = make_uint2(ts.v1, i);
    }
  }
  if (MODE == 0 && lane == 0 && cand_sum) atomicAdd(cand_total, (unsigned long long)cand_sum);
}

// Both passes in one (the resident path): blocks of targets take tickets in
// order, count their distinct pairs, find their offset by a decoupled look-back
// over the earlier blocks' published counts, and write their pairs -- the same
// output as collect_count + scan + collect_write, with the rep rows and the
// length gathers read once.  status[] (zero before the launch): per block,
// bits 62-63 = 0 not ready / 1 its own count / 2 the prefix through it, bits
// 0-61 the value.  A look-back that waits too long sets *error and the block
// writes nothing.
constexpr unsigned long long kStAgg = 1ull << 62, kStIncl = 2ull << 62;
constexpr unsigned long long kStValue = (1ull << 62) - 1;

__global__ void __launch_bounds__(kPairThreads)
collect_scan_kernel(const uint32_t *__restrict__ rep, const uint32_t *__restrict__ lens,
                    uint32_t n, uint32_t bands, float t, unsigned int *__restrict__ ticket,
                    unsigned long long *__restrict__ status,
                    unsigned long long *__restrict__ cand_total,
                    uint64_t *__restrict__ unique_total, unsigned int *__restrict__ error,
                    uint2 *__restrict__ pairs, uint32_t spin_limit) {
  __shared__ uint32_t tile[kBands * kTargetsPerBlock];
  __shared__ uint32_t vals[kPairThreads / 32][32];
  __shared__ uint32_t toff[kTargetsPerBlock];
  __shared__ unsigned long long excl_sh;
  __shared__ uint32_t blk_sh, ok_sh;
  constexpr uint32_t kPer = kTargetsPerBlock / (kPairThreads / 32);  // targets per warp
  if (threadIdx.x == 0) blk_sh = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint32_t blk = blk_sh, i0 = blk * kTargetsPerBlock;
  const uint32_t nblocks = ceil_div(n, kTargetsPerBlock);
  if (blk >= nblocks) {  // more tickets than blocks: only a check of the wait does this
    if (threadIdx.x == 0) atomicOr(error, 1u);
    return;
  }
  for (uint32_t e = threadIdx.x; e < bands * kTargetsPerBlock; e += kPairThreads) {
    const uint32_t b = e / kTargetsPerBlock, c = e % kTargetsPerBlock;
    tile[e] = (i0 + c < n) ? rep[(size_t)b * n + i0 + c] : 0u;
  }
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  TargetScan ts[kPer];
  uint32_t cand_sum = 0;
#pragma unroll
  for (uint32_t k = 0; k < kPer; ++k) {
    const uint32_t c = warp + k * (kPairThreads / 32), i = i0 + c;
    uint32_t u = 0;
    if (i < n) {
      ts[k] = scan_target(tile, c, i, lens, bands, t, vals[warp]);
      cand_sum += ts[k].cand;
      u = __popc(ts[k].first0) + __popc(ts[k].first1);
    } else {
      ts[k] = TargetScan{0u, 0u, 0u, 0u, 0u};
    }
    if (lane == 0) toff[c] = u;
  }
  __syncthreads();
  if (warp == 0) {
    const uint32_t v = toff[lane];  // the block's 32 targets
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, x, o);
      if (lane >= (uint32_t)o) x += y;
    }
    toff[lane] = x - v;
    const uint32_t agg = __shfl_sync(kFull, x, 31);
    unsigned long long excl = 0;
    uint32_t ok = 1;
    if (blk == 0) {
      if (lane == 0) atomicExch(status, kStIncl | agg);
    } else {
      if (lane == 0) atomicExch(status + blk, kStAgg | agg);
      // warp-wide look-back: lane l reads the status of block j - l (lane 0
      // the nearest), 32 predecessors a round, until one holds an inclusive
      // prefix (before block 0: an inclusive 0)
      for (int64_t j = (int64_t)blk - 1; ok;) {
        const int64_t q = j - (int64_t)lane;
        unsigned long long s = kStIncl;
        if (q >= 0) {
          uint32_t spins = 0;
          for (;;) {
            s = *(volatile unsigned long long *)(status + q);
            if ((s >> 62) != 0) break;
            if (++spins > spin_limit) {  // a predecessor never published
              s = 0;
              break;
            }
          }
        }
        if (__any_sync(kFull, s == 0)) {
          if (lane == 0) atomicOr(error, 1u);
          ok = 0;
          break;
        }
        const uint32_t incl = __ballot_sync(kFull, (s >> 62) == 2);
        // lanes up to the nearest inclusive one (all 32 when there is none)
        const uint32_t upto = incl ? (uint32_t)__ffs(incl) - 1u : 31u;
        unsigned long long val = lane <= upto ? (s & kStValue) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(kFull, val, o);
        excl += val;
        if (incl) break;
        j -= 32;
      }
      if (ok && lane == 0) atomicExch(status + blk, kStIncl | (excl + agg));
    }
    if (lane == 0) {
      if (ok && blk + 1 == nblocks) *unique_total = excl + agg;
      excl_sh = excl;
      ok_sh = ok;
    }
  }
  __syncthreads();
  if (ok_sh) {
    const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (uint32_t k = 0; k < kPer; ++k) {
      const uint32_t c = warp + k * (kPairThreads / 32), i = i0 + c;
      if (i >= n) continue;
      const uint64_t base = excl_sh + toff[c];
      if (ts[k].first0 >> lane & 1u)
        pairs[base + __popc(ts[k].first0 & lt_mask)] = make_uint2(ts[k].v0, i);
      if (ts[k].first1 >> lane & 1u)
        pairs[base + __popc(ts[k].first0) + __popc(ts[k].first1 & lt_mask)] =
            make_uint2(ts[k].v1, i);
    }
  }
  if (lane == 0 && cand_sum) atomicAdd(cand_total, (unsigned long long)cand_sum);
}

int collect_scan(const uint32_t *rep, const uint32_t *lens, uint32_t n, uint32_t bands,
                 uint32_t identity, unsigned int *ticket, unsigned long long *status,
                 unsigned long long *cand_total, uint64_t *unique_total, unsigned int *error,
                 uint2 *pairs, cudaStream_t s, uint32_t spin_limit) {
  if (n == 0) return NGIA_OK;
  const uint32_t nblocks = ceil_div(n, kTargetsPerBlock);
  NGIA_CUDA(cudaMemsetAsync(status, 0, (size_t)nblocks * 8, s));
  collect_scan_kernel<<<nblocks, kPairThreads, 0, s>>>(rep, lens, n, bands,
                                                       identity_threshold(identity), ticket,
                                                       status, cand_total, unique_total, error,
                                                       pairs, spin_limit);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

int collect_count(const uint32_t *rep, const uint32_t *lens, uint32_t n, uint32_t bands,
                  uint32_t identity, uint32_t *ucount, unsigned long long *cand_total,
                  cudaStream_t s) {
  if (n == 0) return NGIA_OK;
  collect_kernel<0><<<ceil_div(n, kTargetsPerBlock), kPairThreads, 0, s>>>(
      rep, lens, n, bands, identity_threshold(identity), ucount, cand_total, nullptr,
      nullptr);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

int collect_write(const uint32_t *rep, const uint32_t *lens, uint32_t n, uint32_t bands,
                  uint32_t identity, const uint64_t *offsets, uint2 *pairs,
                  cudaStream_t s) {
  if (n == 0) return NGIA_OK;
  collect_kernel<1><<<ceil_div(n, kTargetsPerBlock), kPairThreads, 0, s>>>(
      rep, lens, n, bands, identity_threshold(identity), nullptr, nullptr, offsets,
      pairs);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

// ---- width classes ------------------------------------------------------------------
constexpr uint32_t kClassifyUnroll = 4;

__global__ void __launch_bounds__(256)
classify_kernel(const uint32_t *__restrict__ lens, const uint2 *__restrict__ pairs,
                uint64_t count, float t, int fma_mode, ClassPlan plan,
                uint32_t *__restrict__ cls,
                unsigned int *__restrict__ class_count,
                unsigned long long *__restrict__ cells) {
  __shared__ unsigned int sc[kNumClasses];
  __shared__ unsigned long long scells;
  if (threadIdx.x < kNumClasses) sc[threadIdx.x] = 0;
  if (threadIdx.x == 0) scells = 0;
  __syncthreads();
  unsigned long long my_cells = 0;
  const uint32_t lt_mask = (1u << (threadIdx.x & 31u)) - 1u;
  // block-uniform trips of kClassifyUnroll pairs per thread (their loads in
  // flight together), so that the class counts can be summed per warp
  constexpr uint32_t U = kClassifyUnroll;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t p0 = (uint64_t)blockIdx.x * blockDim.x; p0 < count; p0 += U * stride) {
    uint2 pr[U];
#pragma unroll
    for (uint32_t u = 0; u < U; ++u) {
      const uint64_t p = p0 + u * stride + threadIdx.x;
      pr[u] = p < count ? pairs[p] : make_uint2(kFull, kFull);
    }
    uint32_t lr[U], lt[U];
#pragma unroll
    for (uint32_t u = 0; u < U; ++u) {
      const bool real = pr[u].x != kFull;
      lr[u] = real ? __ldg(lens + pr[u].x) : 0u;
      lt[u] = real ? __ldg(lens + pr[u].y) : 0u;
    }
#pragma unroll
    for (uint32_t u = 0; u < U; ++u) {
      const uint64_t p = p0 + u * stride + threadIdx.x;
      uint32_t c = kFull;
      if (p < count) {
        if (pr[u].x == kFull) {  // an empty pair slot (serving): never aligned
          c = kSkipClass;
          cls[p] = skip_sort_key();
        } else {
          const Band b = make_band(lr[u], lt[u], t, fma_mode);
          c = (uint32_t)width_class(b, plan);
          cls[p] = class_sort_key((int)c, b);
          my_cells += band_blocks(b);
        }
      }
      const uint32_t peers = __match_any_sync(kFull, c);
      if (c != kFull && (peers & lt_mask) == 0) atomicAdd(&sc[c], (unsigned int)__popc(peers));
    }
  }
  atomicAdd(&scells, my_cells);
  __syncthreads();
  if (threadIdx.x < kNumClasses && sc[threadIdx.x]) atomicAdd(&class_count[threadIdx.x], sc[threadIdx.x]);
  if (threadIdx.x == 0 && scells) atomicAdd(cells, scells * 1024ull);
}

__global__ void class_bounds_kernel(const unsigned int *__restrict__ class_count,
                                    uint32_t *__restrict__ bounds) {
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int c = 0; c < kNumClasses; ++c) {
      bounds[c] = run;
      run += class_count[c];
    }
    bounds[kNumClasses] = run;
  }
}

int classify(const uint32_t *lens, const uint2 *pairs, uint32_t count, uint32_t identity,
             const ClassPlan &plan, uint32_t *cls, unsigned int *class_count,
             unsigned long long *cells, uint32_t *bounds, cudaStream_t s) {
  if (count > 0) {
    int dev = 0, sms = 0;
    NGIA_CUDA(cudaGetDevice(&dev));
    NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const uint32_t want = ceil_div(count, 256u), cap = (uint32_t)sms * 8;
    classify_kernel<<<want < cap ? want : cap, 256, 0, s>>>(
        lens, pairs, count, identity_threshold(identity), round_mode(), plan, cls,
        class_count, cells);
    NGIA_LAUNCHED();
  }
  class_bounds_kernel<<<1, 32, 0, s>>>(class_count, bounds);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

// ---- shares of the pairs by band cells (a graph build split over devices) ----------
// Band blocks of every pair (the reference's visited 32x32 blocks; 0 for a
// pair failing the length filter).
__global__ void __launch_bounds__(256)
pair_blocks_kernel(const uint32_t *__restrict__ lens, const uint2 *__restrict__ pairs,
                   uint32_t count, float t, int fma_mode, uint32_t *__restrict__ blocks) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < count;
       p += gridDim.x * blockDim.x) {
    const uint2 pr = pairs[p];
    const uint64_t b = band_blocks(make_band(__ldg(lens + pr.x), __ldg(lens + pr.y), t, fma_mode));
    blocks[p] = b < kFull ? (uint32_t)b : kFull;
  }
}

// cut[k] for k = part, part + 1: the first pair whose exclusive prefix of
// blocks reaches total * k / parts (0 and count at the ends).
__global__ void part_cut_kernel(const uint64_t *__restrict__ prefix, uint32_t count,
                                const uint64_t *__restrict__ total, uint32_t part, uint32_t parts,
                                uint32_t *__restrict__ cut) {
  const uint32_t k = part + threadIdx.x;
  if (threadIdx.x > 1) return;
  uint32_t c;
  if (k == 0) {
    c = 0;
  } else if (k >= parts) {
    c = count;
  } else {
    const uint64_t target = *total / parts * k + (*total % parts) * k / parts;
    uint32_t lo = 0, hi = count;  // first index with prefix >= target
    while (lo < hi) {
      const uint32_t mid = lo + (hi - lo) / 2;
      if (prefix[mid] < target) lo = mid + 1; else hi = mid;
    }
    c = lo;
  }
  cut[threadIdx.x] = c;
}

size_t share_scratch_bytes(uint32_t count) {
  const size_t c = count ? count : 1;
  return c * 4 + c * 8 + scan_scratch_bytes(count) + 64;
}

int share_range(const uint32_t *lens, const uint2 *pairs, uint32_t count, uint32_t identity,
                uint32_t part, uint32_t parts, void *scratch, uint32_t h_cut[2],
                cudaStream_t s) {
  if (parts <= 1 || count == 0) {
    h_cut[0] = 0;
    h_cut[1] = count;
    return NGIA_OK;
  }
  char *w = static_cast<char *>(scratch);
  const size_t c = count;
  uint32_t *blocks = reinterpret_cast<uint32_t *>(w);
  uint64_t *prefix = reinterpret_cast<uint64_t *>(w + ((c * 4 + 15) & ~(size_t)15));
  uint64_t *total = prefix + c;
  uint32_t *cut = reinterpret_cast<uint32_t *>(total + 1);
  void *scan_tmp = cut + 4;
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint32_t want = ceil_div(count, 256u), cap = (uint32_t)sms * 8u;
  pair_blocks_kernel<<<want < cap ? want : cap, 256, 0, s>>>(
      lens, pairs, count, identity_threshold(identity), round_mode(), blocks);
  NGIA_LAUNCHED();
  NGIA_TRY(exclusive_scan_u64(blocks, prefix, count, total, scan_tmp, s));
  part_cut_kernel<<<1, 32, 0, s>>>(prefix, count, total, part, parts, cut);
  NGIA_LAUNCHED();
  NGIA_CUDA(cudaMemcpyAsync(h_cut, cut, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  return NGIA_OK;
}

// ---- emission -----------------------------------------------------------------------
__global__ void __launch_bounds__(256)
positive_flags_kernel(const uint32_t *__restrict__ scores, uint32_t stride, uint32_t count,
                      uint32_t *__restrict__ flags) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < count) flags[p] = scores[(size_t)p * stride] > 0 ? 1u : 0u;
}

// Ordered compaction of the pairs with score > 0 in three passes that touch
// the scores twice and nothing per pair besides: per-block counts over runs
// of kEmitRun pairs, their exclusive scan (one block), then each block writes
// its hits from its offset in pair order (ballots within a warp, warp counts
// across the block).
constexpr uint32_t kEmitRun = 4096;

__global__ void __launch_bounds__(256)
count_hits_kernel(const uint32_t *__restrict__ scores, uint32_t count,
                  uint32_t *__restrict__ bcount) {
  __shared__ uint32_t wsum[8];
  const uint32_t beg = blockIdx.x * kEmitRun, end = min(beg + kEmitRun, count);
  uint32_t c = 0;
  for (uint32_t p = beg + threadIdx.x; p < end; p += 256) c += scores[p] > 0 ? 1u : 0u;
  c = __reduce_add_sync(kFull, c);
  if ((threadIdx.x & 31u) == 0) wsum[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < 8; ++w) t += wsum[w];
    bcount[blockIdx.x] = t;
  }
}

// exclusive scan of nb counts in place (one block of 1024), total -> *m
__global__ void __launch_bounds__(1024)
scan_hits_kernel(uint32_t *__restrict__ b, uint32_t nb, uint64_t *__restrict__ m) {
  __shared__ uint32_t part[32];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t run = 0;
  for (uint32_t base = 0; base < nb; base += 1024) {  // block-uniform
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < nb ? b[i] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int k = 1; k < 32; k <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, x, k);
      if (lane >= (uint32_t)k) x += y;
    }
    if (lane == 31) part[warp] = x;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (uint32_t w = 0; w < 32; ++w) {
      before += w < warp ? part[w] : 0u;
      total += part[w];
    }
    if (i < nb) b[i] = run + before + x - v;
    run += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) *m = run;
}

__global__ void __launch_bounds__(256)
compact_hits_kernel(const uint2 *__restrict__ pairs, const uint32_t *__restrict__ scores,
                    uint32_t count, const uint32_t *__restrict__ boff,
                    uint32_t *__restrict__ erep, uint32_t *__restrict__ etar,
                    uint32_t *__restrict__ escore) {
  __shared__ uint32_t wsum[8];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t beg = blockIdx.x * kEmitRun, end = min(beg + kEmitRun, count);
  uint32_t run = boff[blockIdx.x];
  for (uint32_t p0 = beg; p0 < end; p0 += 256) {  // block-uniform
    const uint32_t p = p0 + threadIdx.x;
    const uint32_t sc = p < end ? scores[p] : 0u;
    const uint32_t hits = __ballot_sync(kFull, sc > 0);
    if (lane == 0) wsum[warp] = __popc(hits);
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (uint32_t w = 0; w < 8; ++w) {
      before += w < warp ? wsum[w] : 0u;
      total += wsum[w];
    }
    if (sc > 0) {
      const uint32_t e = run + before + __popc(hits & ((1u << lane) - 1u));
      const uint2 pr = pairs[p];
      erep[e] = pr.x;
      etar[e] = pr.y;
      escore[e] = sc;
    }
    run += total;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256)
gather_edges_kernel(const uint32_t *__restrict__ srep, const uint32_t *__restrict__ sidx,
                    const uint32_t *__restrict__ etar, const uint32_t *__restrict__ escore,
                    uint32_t m, ngia_edge *__restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const uint32_t e = sidx[k];
  ngia_edge ed;
  ed.rep = (int32_t)srep[k];
  ed.tar = (int32_t)etar[e];
  ed.weight = __fdiv_rn(__uint2float_rn(escore[e]), 100.0f);
  out[k] = ed;
}

// Job triples with score > 0 -> edges in job order.
__global__ void __launch_bounds__(256)
jobs_to_edges_kernel(const uint32_t *__restrict__ jobs, uint32_t count,
                     const uint64_t *__restrict__ off, ngia_edge *__restrict__ out) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= count) return;
  const uint32_t sc = jobs[3 * (size_t)j + 2];
  if (sc == 0) return;
  ngia_edge ed;
  ed.rep = (int32_t)jobs[3 * (size_t)j];
  ed.tar = (int32_t)jobs[3 * (size_t)j + 1];
  ed.weight = __fdiv_rn(__uint2float_rn(sc), 100.0f);
  out[off[j]] = ed;
}

__global__ void store_u32_from_u64_kernel(const uint64_t *src, uint32_t *dst) { *dst = (uint32_t)*src; }

int bits_for(uint32_t max_value) {
  int b = 0;
  while (b < 32 && (max_value >> b) != 0) ++b;
  return b;
}

size_t emit_scratch_bytes(uint32_t count, uint32_t n_nodes) {
  (void)n_nodes;
  const size_t c = count ? count : 1;
  // flags + offsets + 3 compacted arrays + 2 sorted arrays + sort scratch + scan
  return c * 4 + c * 8 + 3 * c * 4 + 2 * c * 4 + radix_sort_scratch_bytes(count, 1) +
         scan_scratch_bytes(count) + 64;
}

// Pairs (target order) with scores -> edges sorted by (rep, tar).  Sorting the
// target-ordered list stably by rep gives (rep, tar) order.  *h_m = edges.
int emit_sorted(const uint2 *pairs, const uint32_t *scores, uint32_t count,
                uint32_t n_nodes, ngia_edge *out, uint64_t *h_m, void *scratch,
                cudaStream_t s) {
  *h_m = 0;
  if (count == 0) return NGIA_OK;
  char *w = static_cast<char *>(scratch);
  uint32_t *flags = reinterpret_cast<uint32_t *>(w);
  w += (size_t)count * 4;
  uint64_t *off = reinterpret_cast<uint64_t *>((reinterpret_cast<uintptr_t>(w) + 15) & ~uintptr_t(15));
  w = reinterpret_cast<char *>(off + count);
  uint32_t *erep = reinterpret_cast<uint32_t *>(w);
  uint32_t *etar = erep + count;
  uint32_t *escore = etar + count;
  uint32_t *srep = escore + count;
  uint32_t *sidx = srep + count;
  char *sort_scratch = reinterpret_cast<char *>(sidx + count);
  uint64_t *scan_tmp = reinterpret_cast<uint64_t *>(
      (reinterpret_cast<uintptr_t>(sort_scratch + radix_sort_scratch_bytes(count, 1)) + 15) &
      ~uintptr_t(15));
  uint64_t *d_total = scan_tmp + ceil_div<size_t>(count, 2048) + 1;
  (void)off;
  const uint32_t runs = ceil_div(count, kEmitRun);
  uint32_t *bcount = flags;  // runs words (count >= runs)
  count_hits_kernel<<<runs, 256, 0, s>>>(scores, count, bcount);
  NGIA_LAUNCHED();
  scan_hits_kernel<<<1, 1024, 0, s>>>(bcount, runs, d_total);
  NGIA_LAUNCHED();
  compact_hits_kernel<<<runs, 256, 0, s>>>(pairs, scores, count, bcount, erep, etar, escore);
  NGIA_LAUNCHED();
  uint64_t m = 0;
  NGIA_CUDA(cudaMemcpyAsync(&m, d_total, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  *h_m = m;
  if (m == 0) return NGIA_OK;
  const int bits = bits_for(n_nodes ? n_nodes - 1 : 0);
  NGIA_TRY(radix_sort_pairs(erep, nullptr, srep, sidx, (uint32_t)m, 1, 0,
                            bits > 0 ? bits : 8, sort_scratch, s));
  gather_edges_kernel<<<ceil_div((uint32_t)m, 256u), 256, 0, s>>>(srep, sidx, etar, escore,
                                                                  (uint32_t)m, out);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

// ---- fast mode ------------------------------------------------------------------------
// Jobs of one band (src/fastClustering.hpp:256-258): rep[i] != i and i not
// yet assigned.  The order of jobs inside a band does not affect the result
// (each target appears once per band), so they are appended with one atomic
// per warp.
__global__ void __launch_bounds__(256)
fast_jobs_kernel(const uint32_t *__restrict__ rep_row, const uint32_t *__restrict__ parent,
                 uint32_t n, uint32_t *__restrict__ jobs, uint32_t *__restrict__ d_count) {
  const uint32_t lane = threadIdx.x & 31u;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t r = i < n ? rep_row[i] : 0u;
    const bool job = i < n && r != i && parent[i] == kFull;
    const uint32_t bal = __ballot_sync(kFull, job);
    uint32_t slot = 0;
    if (lane == 0 && bal) slot = atomicAdd(d_count, (uint32_t)__popc(bal));
    slot = __shfl_sync(kFull, slot, 0) + __popc(bal & ((1u << lane) - 1u));
    if (job) {
      jobs[3 * (size_t)slot] = r;
      jobs[3 * (size_t)slot + 1] = i;
      jobs[3 * (size_t)slot + 2] = 0;
    }
  }
}

// A hit assigns the target to its rep (src/fastClustering.hpp:330-334).
__global__ void __launch_bounds__(256)
fast_assign_kernel(const uint32_t *__restrict__ jobs, const uint32_t *__restrict__ d_count,
                   uint32_t *__restrict__ parent) {
  const uint32_t count = *d_count;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count;
       j += gridDim.x * blockDim.x)
    if (jobs[3 * (size_t)j + 2] > 0) parent[jobs[3 * (size_t)j + 1]] = jobs[3 * (size_t)j];
}

int fast_round(const uint32_t *packed, const uint64_t *offs, const uint32_t *rep_row,
               uint32_t *parent, uint32_t n, uint32_t identity, uint32_t *jobs,
               uint32_t *d_count, cudaStream_t s) {
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  NGIA_CUDA(cudaMemsetAsync(d_count, 0, sizeof(uint32_t), s));
  const uint32_t want = ceil_div(n, 256u), cap = (uint32_t)sms * 8;
  fast_jobs_kernel<<<want < cap ? want : cap, 256, 0, s>>>(rep_row, parent, n, jobs, d_count);
  NGIA_LAUNCHED();
  NGIA_TRY(launch_align_jobs_dev_count(packed, offs, jobs, d_count, n, identity, s));
  fast_assign_kernel<<<want < cap ? want : cap, 256, 0, s>>>(jobs, d_count, parent);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

}  // namespace ngia

extern "C" int ngia_emit_edges(const uint32_t *d_jobs, uint32_t count, ngia_edge *d_edges,
                               uint32_t *d_n_edges, void *stream) {
  using namespace ngia;
  if (!d_n_edges) return NGIA_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (count == 0) {
    NGIA_CUDA(cudaMemsetAsync(d_n_edges, 0, sizeof(uint32_t), s));
    return NGIA_OK;
  }
  if (!d_jobs || !d_edges) return NGIA_ERR_ARG;
  const size_t bytes = (size_t)count * 4 + (size_t)count * 8 + scan_scratch_bytes(count) + 64;
  void *scratch = nullptr;
  cudaError_t e = cudaMallocAsync(&scratch, bytes, s);
  if (e != cudaSuccess) {
    cuda_fail(e);
    return NGIA_ERR_NOMEM;
  }
  uint32_t *flags = static_cast<uint32_t *>(scratch);
  uint64_t *off = reinterpret_cast<uint64_t *>(
      (reinterpret_cast<uintptr_t>(flags + count) + 15) & ~uintptr_t(15));
  uint64_t *scan_tmp = off + count;
  uint64_t *d_total = scan_tmp + ceil_div<size_t>(count, 2048) + 1;
  int st = NGIA_OK;
  const uint32_t blocks = ceil_div(count, 256u);
  positive_flags_kernel<<<blocks, 256, 0, s>>>(d_jobs + 2, 3, count, flags);
  note_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) st = cuda_fail(e);
  if (st == NGIA_OK) st = exclusive_scan_u64(flags, off, count, d_total, scan_tmp, s);
  if (st == NGIA_OK) {
    jobs_to_edges_kernel<<<blocks, 256, 0, s>>>(d_jobs, count, off, d_edges);
    note_launch();
    store_u32_from_u64_kernel<<<1, 1, 0, s>>>(d_total, d_n_edges);
    note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) st = cuda_fail(e);
  }
  e = cudaFreeAsync(scratch, s);
  if (st == NGIA_OK && e != cudaSuccess) st = cuda_fail(e);
  return st;
}
