// align.cu -- alignment kernels: the drop-in job-triple kernel and the
// length-binned batched kernels.
#include <mutex>
#include <vector>

#include "align.cuh"
#include "align_group.cuh"
#include "align_group_cta.cuh"
#include "align_stream.cuh"
#include "kernels.cuh"

namespace ngia {

// One thread per job, in job order: the drop-in for the reference's
// one-launch-per-band kernel_dynamic<<<ceil(count/64), 64>>> (launch at
// src/buildGraph.hpp:323).  The window width is picked per pair at run time.
__device__ __forceinline__ uint32_t lcs_any(const uint32_t *rep, const uint32_t *tar,
                                            const Band &b, uint32_t *lines) {
  uint32_t blocks;
  if (b.width <= 4) return lcs_window<4>(rep, tar, b, blocks);
  if (b.width <= 8) return lcs_window<8>(rep, tar, b, blocks);
  if (b.width <= 16) return lcs_window<16>(rep, tar, b, blocks);
  return lcs_general(rep, tar, b, lines, blocks);
}

// Adds the warp's computed 32x32 blocks (row words x column blocks) to *work.
__device__ __forceinline__ void count_work(uint32_t blocks, unsigned long long *work) {
  // two 16-bit halves, so that a warp's sum cannot overflow
  const uint32_t lo = __reduce_add_sync(kFull, blocks & 0xFFFFu);
  const uint32_t hi = __reduce_add_sync(kFull, blocks >> 16);
  const unsigned long long sum = ((unsigned long long)hi << 16) + lo;
  if ((threadIdx.x & 31u) == 0 && sum) atomicAdd(work, sum);
}

__global__ void __launch_bounds__(128)
align_jobs_kernel(const uint32_t *__restrict__ packed,
                  const uint64_t *__restrict__ offs, uint32_t *__restrict__ jobs,
                  uint32_t count, float t, int fma_mode) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= count) return;
  const uint32_t *rep = packed + offs[jobs[3 * j]];
  const uint32_t *tar = packed + offs[jobs[3 * j + 1]];
  const uint32_t lr = __ldg(rep), lt = __ldg(tar);
  const Band b = make_band(lr, lt, t, fma_mode);
  if (!b.pass) return;  // the reference leaves the score word as it was
  uint32_t lines[kMaxRowBlocks];
  const uint32_t lcs = lcs_any(rep, tar, b, lines);
  jobs[3 * j + 2] = identity_score(lcs, lr, lt, t);
}

// Same over a job list whose length lives in device memory (graph-capturable
// per-band rounds of fast mode).  Grid-stride.
__global__ void __launch_bounds__(128)
align_jobs_dev_count_kernel(const uint32_t *__restrict__ packed,
                            const uint64_t *__restrict__ offs,
                            uint32_t *__restrict__ jobs,
                            const uint32_t *__restrict__ d_count, float t,
                            int fma_mode) {
  const uint32_t count = *d_count;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < count;
       j += gridDim.x * blockDim.x) {
    const uint32_t *rep = packed + offs[jobs[3 * j]];
    const uint32_t *tar = packed + offs[jobs[3 * j + 1]];
    const uint32_t lr = __ldg(rep), lt = __ldg(tar);
    const Band b = make_band(lr, lt, t, fma_mode);
    if (!b.pass) continue;
    uint32_t lines[kMaxRowBlocks];
    const uint32_t lcs = lcs_any(rep, tar, b, lines);
    jobs[3 * j + 2] = identity_score(lcs, lr, lt, t);
  }
}

// The batched kernels read their class's range of the queue order from
// device memory (bounds[cls] .. bounds[cls + 1], written by the classifier),
// so that a round needs no host round trip and can be captured as a graph.

// Batched form, general kernel: one pair per thread, grid-stride over the
// class's range.
__global__ void __launch_bounds__(128)
align_general_kernel(const uint32_t *__restrict__ packed,
                     const uint64_t *__restrict__ offs, const uint2 *__restrict__ pairs,
                     const uint32_t *__restrict__ order, const uint32_t *__restrict__ bounds,
                     int cls, uint32_t *__restrict__ scores, float t, int fma_mode,
                     unsigned long long *__restrict__ work) {
  const uint32_t begin = bounds[cls], end = bounds[cls + 1];
  uint32_t done = 0;
  for (uint32_t k = begin + blockIdx.x * blockDim.x + threadIdx.x; k < end;
       k += gridDim.x * blockDim.x) {
    const uint32_t p = order[k];
    const uint2 pr = pairs[p];
    const uint32_t *rep = packed + offs[pr.x];
    const uint32_t *tar = packed + offs[pr.y];
    const uint32_t lr = __ldg(rep), lt = __ldg(tar);
    const Band b = make_band(lr, lt, t, fma_mode);
    uint32_t lines[kMaxRowBlocks];
    uint32_t blocks;
    const uint32_t lcs = lcs_general(rep, tar, b, lines, blocks);
    done += blocks * ((b.width + 7u) & ~7u);
    scores[p] = identity_score(lcs, lr, lt, t);
  }
  count_work(done, work);
}

// Batched form, group kernel (align_group.cuh): a persistent grid whose groups
// of G lanes take pairs of one class from its queue.
template <int G, int K, int KC>
__global__ void __launch_bounds__(kGroupThreads)
align_group_kernel(const uint32_t *__restrict__ packed, const uint32_t *__restrict__ nib,
                   uint64_t inv, const uint64_t *__restrict__ offs,
                   const uint2 *__restrict__ pairs, const uint32_t *__restrict__ order,
                   const uint32_t *__restrict__ bounds, int cls,
                   unsigned int *__restrict__ cursor, uint32_t *__restrict__ scores, float t,
                   int fma_mode, unsigned long long *__restrict__ work) {
  extern __shared__ uint32_t smem[];
  const uint32_t done = align_group<G, K, KC>(packed, nib, inv, offs, pairs, order,
                                              bounds[cls], bounds[cls + 1], cursor, scores, t,
                                              fma_mode, smem);
  count_work(done, work);
}

// The widest group classes: one block of W warps per pair
// (align_group_cta.cuh).
template <int W, int K, int KC>
__global__ void __launch_bounds__(32 * W)
align_group_cta_kernel(const uint32_t *__restrict__ packed, const uint32_t *__restrict__ nib,
                       uint64_t inv, const uint64_t *__restrict__ offs,
                       const uint2 *__restrict__ pairs, const uint32_t *__restrict__ order,
                       const uint32_t *__restrict__ bounds, int cls,
                       unsigned int *__restrict__ cursor, uint32_t *__restrict__ scores, float t,
                       int fma_mode, unsigned long long *__restrict__ work) {
  extern __shared__ uint32_t smem[];
  const uint32_t done = align_group_cta<W, K, KC>(packed, nib, inv, offs, pairs, order,
                                                  bounds[cls], bounds[cls + 1], cursor, scores,
                                                  t, fma_mode, smem);
  count_work(done, work);
}

// Batched form, streaming shared-memory table kernel (align_stream.cuh):
// a persistent grid whose lanes take pairs of one class from its queue.
template <int W, int K>
__global__ void __launch_bounds__(kStreamThreads, NGIA_STREAM_MIN_BLOCKS)
align_stream_kernel(const uint32_t *__restrict__ packed, const uint32_t *__restrict__ nib,
                    uint64_t inv, const uint64_t *__restrict__ offs,
                    const uint2 *__restrict__ pairs, const uint32_t *__restrict__ order,
                    const uint32_t *__restrict__ bounds, int cls,
                    unsigned int *__restrict__ cursor, uint32_t *__restrict__ scores, float t,
                    int fma_mode, unsigned long long *__restrict__ work) {
  extern __shared__ uint32_t smem[];
  const uint32_t done = align_stream<W, K>(packed, nib, inv, offs, pairs, order, bounds[cls],
                                           bounds[cls + 1], cursor, scores, t, fma_mode, smem);
  count_work(done, work);
}

// Load-time layout kernels: one warp per record, lane k taking the record's
// 32-residue blocks k, k + 32, ... (four words each, coalesced across the
// warp); bit work by shifts and masks, no per-residue loops.

// bits 0..7 of b to bits 0, 4, ..., 28
__device__ __forceinline__ uint32_t spread8(uint32_t b) {
  b = (b | (b << 12)) & 0x000F000Fu;
  b = (b | (b << 6)) & 0x03030303u;
  return (b | (b << 3)) & 0x11111111u;
}

// Four plane words of a block (bit r of plane e = bit e of the code of
// residue r) -> its four nibble words (word q: residues 8q..8q+7, the first in
// the high nibble).
__device__ __forceinline__ void planes_to_nibbles(const uint32_t (&pl)[4], int np,
                                                  uint32_t (&out)[4]) {
  uint32_t rv[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) rv[e] = e < np ? __brev(pl[e]) : 0u;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t w = 0;
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (e < np) w |= spread8((rv[e] >> (24 - 8 * q)) & 0xFFu) << e;
    out[q] = w;
  }
}

// mask of the residues of a block whose code is c, from its four planes
__device__ __forceinline__ uint32_t code_mask(const uint32_t (&pl)[4], uint32_t c) {
  return ((c & 1u) ? pl[0] : ~pl[0]) & ((c & 2u) ? pl[1] : ~pl[1]) &
         ((c & 4u) ? pl[2] : ~pl[2]) & ((c & 8u) ? pl[3] : ~pl[3]);
}

// Planes -> nibbles: the same record layout, with each block's four plane
// words replaced by four words of eight 4-bit codes.  The length word is
// copied.  presence |= bit c for every code c of a real residue.  A record
// whose offset lies outside the `words` of the region, whose length word is
// not lens[i], or whose blocks run past the region is left alone and sets
// kBadRecord in presence.
__global__ void __launch_bounds__(256)
nibble_kernel(const uint32_t *__restrict__ packed, const uint64_t *__restrict__ offs,
              const uint32_t *__restrict__ lens, uint32_t n, uint64_t words,
              uint32_t *__restrict__ nib, uint32_t *__restrict__ presence) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  uint32_t mine = 0;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const uint64_t o = offs[i];
    if (o >= words) {
      mine |= kBadRecord;
      continue;
    }
    const uint32_t len = __ldg(packed + o);
    if (len != lens[i] || o + 1 + 4ull * ((len + 31) >> 5) > words) {
      // flagged; an empty record in its place, so that a kernel reading the
      // layout before the flag is seen stays inside the region
      if (lane == 0) nib[o] = 0;
      mine |= kBadRecord;
      continue;
    }
    if (lane == 0) nib[o] = len;
    const uint32_t blocks = (len + 31) >> 5;
    for (uint32_t k = lane; k < blocks; k += 32) {
      const uint32_t *src = packed + o + 1 + 4 * k;
      const uint32_t pl[4] = {__ldg(src), __ldg(src + 1), __ldg(src + 2), __ldg(src + 3)};
      uint32_t w[4];
      planes_to_nibbles(pl, 4, w);
      uint32_t *dst = nib + o + 1 + 4 * k;
#pragma unroll
      for (int q = 0; q < 4; ++q) dst[q] = w[q];
      const uint32_t left = len - 32 * k;
      const uint32_t real = left >= 32 ? kFull : (1u << left) - 1u;
#pragma unroll
      for (uint32_t c = 0; c < 16; ++c)
        if (code_mask(pl, c) & real) mine |= 1u << c;
    }
  }
  mine = __reduce_or_sync(kFull, mine);
  if (lane == 0 && mine) atomicOr(presence, mine);
}

// Recoded databases from their packed planes, in one pass: the aligner-code
// nibbles (each residue code c replaced by map nibble c) and the planes of the aligner codes
// (planes 0-2, plane 3 zero).  bits[b] = the residue codes whose aligner code
// has bit b set.
__global__ void __launch_bounds__(256)
dense_layouts_kernel(const uint32_t *__restrict__ packed, const uint64_t *__restrict__ offs,
                     uint32_t n, uint32_t bit0, uint32_t bit1, uint32_t bit2,
                     uint32_t *__restrict__ dense_nib, uint32_t *__restrict__ dplanes) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const uint64_t o = offs[i];
    const uint32_t len = __ldg(packed + o);
    if (lane == 0) {
      dense_nib[o] = len;
      dplanes[o] = len;
    }
    const uint32_t blocks = (len + 31) >> 5;
    for (uint32_t k = lane; k < blocks; k += 32) {
      const uint32_t *src = packed + o + 1 + 4 * k;
      const uint32_t pl[4] = {__ldg(src), __ldg(src + 1), __ldg(src + 2), __ldg(src + 3)};
      uint32_t d[4] = {0u, 0u, 0u, 0u};
#pragma unroll
      for (uint32_t c = 1; c < 16; ++c) {
        const uint32_t m = code_mask(pl, c);
        d[0] |= (bit0 >> c) & 1u ? m : 0u;
        d[1] |= (bit1 >> c) & 1u ? m : 0u;
        d[2] |= (bit2 >> c) & 1u ? m : 0u;
      }
      uint32_t w[4];
      planes_to_nibbles(d, 3, w);
      uint32_t *dn = dense_nib + o + 1 + 4 * k, *dp = dplanes + o + 1 + 4 * k;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        dn[q] = w[q];
        dp[q] = d[q];
      }
    }
  }
}

int launch_nibbles(const uint32_t *packed, const uint64_t *offs, const uint32_t *lens,
                   uint32_t n, uint64_t words, uint32_t *nib, uint32_t *presence, cudaStream_t s,
                   bool accumulate) {
  if (n == 0) return NGIA_OK;
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint32_t want = ceil_div(n, 8u), cap = (uint32_t)sms * 16u;
  if (!accumulate) NGIA_CUDA(cudaMemsetAsync(presence, 0, sizeof(uint32_t), s));
  nibble_kernel<<<want < cap ? want : cap, 256, 0, s>>>(packed, offs, lens, n, words, nib,
                                                        presence);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

// The layouts a recoded database needs, for a run of records in one pass over
// their planes, for loads whose code map is assumed ahead (the pipelined
// load): recoded nibbles and code planes (the sketch reads residue codes from
// the planes themselves).  Only the map's own codes are looked at: a residue
// of another code (or a record outside words [w0, w1), which is then left
// empty) sets *bad, and the load falls back.  Any subset of the map's codes
// is served by the same map (it stays one-to-one on the codes present).
// codes[k], k < ncodes: the residue codes of the map, aligner code k + 1.
// kDense / kPlanes: which of the two layouts a launch writes (a null output
// pointer leaves its layout out).
template <bool kDense, bool kPlanes>
__global__ void __launch_bounds__(256)
load_layouts_kernel(const uint32_t *__restrict__ packed, const uint64_t *__restrict__ offs,
                    const uint32_t *__restrict__ lens, uint32_t n, uint64_t w0, uint64_t w1,
                    uint64_t words, uint32_t codes, uint32_t ncodes,
                    uint32_t *__restrict__ dense_nib, uint32_t *__restrict__ dplanes,
                    uint32_t *__restrict__ bad) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  bool wrong = false;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const uint64_t o = offs[i];
    // a record outside its piece or with the wrong length word is flagged and,
    // when its offset lies in the region, left empty in every layout (the
    // sketch also bounds every record it reads by the region)
    if (o < w0 || o >= w1) {
      if (lane == 0 && o < words) {
        if (kDense) dense_nib[o] = 0;
        if (kPlanes) dplanes[o] = 0;
      }
      wrong = true;
      continue;
    }
    const uint32_t len = __ldg(packed + o);
    const uint32_t blocks = (len + 31) >> 5;
    if (len != lens[i] || o + 1 + 4ull * blocks > w1) {
      if (lane == 0) {
        if (kDense) dense_nib[o] = 0;
        if (kPlanes) dplanes[o] = 0;
      }
      wrong = true;
      continue;
    }
    if (lane == 0) {
      if (kDense) dense_nib[o] = len;
      if (kPlanes) dplanes[o] = len;
    }
    for (uint32_t k = lane; k < blocks; k += 32) {
      const uint64_t b = o + 1 + 4ull * k;
      const uint32_t pl[4] = {__ldg(packed + b), __ldg(packed + b + 1), __ldg(packed + b + 2),
                              __ldg(packed + b + 3)};
      const uint32_t left = len - 32 * k;
      const uint32_t real = left >= 32 ? kFull : (1u << left) - 1u;
      uint32_t d[4] = {0u, 0u, 0u, 0u}, known = 0u;
      for (uint32_t j = 0; j < ncodes; ++j) {
        const uint32_t m = code_mask(pl, (codes >> (4 * j)) & 15u);
        const uint32_t a = j + 1;  // aligner code
        known |= m;
        d[0] |= a & 1u ? m : 0u;
        d[1] |= a & 2u ? m : 0u;
        d[2] |= a & 4u ? m : 0u;
      }
      if (real & ~known) wrong = true;
      if (kDense) {
        uint32_t dn[4];
        planes_to_nibbles(d, 3, dn);
#pragma unroll
        for (int q = 0; q < 4; ++q) dense_nib[b + q] = dn[q];
      }
      if (kPlanes) {
#pragma unroll
        for (int q = 0; q < 4; ++q) dplanes[b + q] = d[q];
      }
    }
  }
  if (__ballot_sync(kFull, wrong) && lane == 0) atomicOr(bad, 1u);
}

static int map_bits(uint64_t map, uint32_t (&bits)[3]) {
  bits[0] = bits[1] = bits[2] = 0u;
  for (uint32_t c = 1; c < 16; ++c) {
    const uint32_t d = (uint32_t)(map >> (4 * c)) & 15u;
    if (d > 7) return NGIA_ERR_ARG;  // three planes hold aligner codes 0..7
    for (int b = 0; b < 3; ++b)
      if ((d >> b) & 1u) bits[b] |= 1u << c;
  }
  return NGIA_OK;
}

int launch_load_layouts(const uint32_t *packed, const uint64_t *offs, const uint32_t *lens,
                        uint32_t n, uint64_t w0, uint64_t w1, uint64_t words, uint64_t inv,
                        uint32_t *dense_nib, uint32_t *dplanes, uint32_t *bad,
                        cudaStream_t s) {
  if (w0 > w1 || w1 > words) return NGIA_ERR_ARG;
  if (n == 0) return NGIA_OK;
  uint32_t codes = 0, ncodes = 0;  // inv nibble d = residue code of aligner code d
  for (uint32_t d = 1; d < 8; ++d) {
    const uint32_t c = (uint32_t)(inv >> (4 * d)) & 15u;
    if (c == 0) break;
    codes |= c << (4 * ncodes++);
  }
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint32_t want = ceil_div(n, 8u), cap = (uint32_t)sms * 16u;
  if (!dense_nib && !dplanes) return NGIA_OK;
  if (dense_nib && dplanes)
    load_layouts_kernel<true, true><<<want < cap ? want : cap, 256, 0, s>>>(
        packed, offs, lens, n, w0, w1, words, codes, ncodes, dense_nib, dplanes, bad);
  else if (dense_nib)
    load_layouts_kernel<true, false><<<want < cap ? want : cap, 256, 0, s>>>(
        packed, offs, lens, n, w0, w1, words, codes, ncodes, dense_nib, dplanes, bad);
  else
    load_layouts_kernel<false, true><<<want < cap ? want : cap, 256, 0, s>>>(
        packed, offs, lens, n, w0, w1, words, codes, ncodes, dense_nib, dplanes, bad);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

int launch_dense_layouts(const uint32_t *packed, const uint64_t *offs, uint32_t n,
                         uint64_t map, uint32_t *dense_nib, uint32_t *dplanes,
                         cudaStream_t s) {
  if (n == 0) return NGIA_OK;
  uint32_t bits[3];
  NGIA_TRY(map_bits(map, bits));
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint32_t want = ceil_div(n, 8u), cap = (uint32_t)sms * 16u;
  dense_layouts_kernel<<<want < cap ? want : cap, 256, 0, s>>>(packed, offs, n, bits[0], bits[1],
                                                               bits[2], dense_nib, dplanes);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

// Blocks of a persistent launch: as many as fit on the device at once, and no
// more than `want`.  Occupancy is looked up once per (kernel, device).
struct OccEntry {
  const void *func;
  int dev, per_sm, sms;
};
static std::mutex g_occ_mu;
static std::vector<OccEntry> g_occ;

template <typename F>
static int persistent_grid(F func, int threads, size_t smem, uint32_t want, uint32_t *grid) {
  int dev = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  const void *key = reinterpret_cast<const void *>(func);
  std::lock_guard<std::mutex> lock(g_occ_mu);
  const OccEntry *hit = nullptr;
  for (const OccEntry &e : g_occ)
    if (e.func == key && e.dev == dev) hit = &e;
  if (!hit) {
    OccEntry e{key, dev, 0, 0};
    NGIA_CUDA(cudaDeviceGetAttribute(&e.sms, cudaDevAttrMultiProcessorCount, dev));
    NGIA_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // the most shared memory per SM the L1 split allows: more resident blocks
    NGIA_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   (int)cudaSharedmemCarveoutMaxShared));
    NGIA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e.per_sm, func, threads, smem));
    if (e.per_sm < 1) e.per_sm = 1;
    g_occ.push_back(e);
    hit = &g_occ.back();
  }
  const uint32_t cap = (uint32_t)(hit->per_sm * hit->sms);
  *grid = want < cap ? want : cap;
  return NGIA_OK;
}

// Launch arguments shared by every class of one batched round.
struct RoundArgs {
  const uint32_t *packed, *nib;
  uint64_t inv;
  const uint32_t *dplanes;
  const uint64_t *offs;
  const uint2 *pairs;
  const uint32_t *order, *bounds;
  uint32_t *scores;
  float t;
  int fm;
  unsigned long long *work;
};

template <int W, int K>
static int launch_stream_k(const RoundArgs &a, int cls, unsigned int *cursor,
                           cudaStream_t s) {
  constexpr size_t smem = stream_smem_bytes(W, K);
  uint32_t grid = 0;
  NGIA_TRY(persistent_grid(align_stream_kernel<W, K>, kStreamThreads, smem, kFull, &grid));
  // K < 16 tables fill from the code planes (records with the same offsets)
  if (K < 16 && !a.dplanes) return NGIA_ERR_STATE;
  align_stream_kernel<W, K><<<grid, kStreamThreads, smem, s>>>(
      K < 16 ? a.dplanes : a.packed, a.nib, a.inv, a.offs, a.pairs, a.order, a.bounds, cls,
      cursor, a.scores, a.t, a.fm, a.work);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

template <int G, int K, int KC>
static int launch_group_k(const RoundArgs &a, int cls, unsigned int *cursor, cudaStream_t s) {
  constexpr size_t smem = group_smem_bytes(K, KC);
  uint32_t grid = 0;
  NGIA_TRY(persistent_grid(align_group_kernel<G, K, KC>, kGroupThreads, smem, kFull, &grid));
  if (KC == 8 && !a.dplanes) return NGIA_ERR_STATE;
  align_group_kernel<G, K, KC><<<grid, kGroupThreads, smem, s>>>(
      KC == 8 ? a.dplanes : a.packed, a.nib, a.inv, a.offs, a.pairs, a.order, a.bounds, cls,
      cursor, a.scores, a.t, a.fm, a.work);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

template <int W, int K, int KC>
static int launch_group_cta_k(const RoundArgs &a, int cls, unsigned int *cursor,
                              cudaStream_t s) {
  constexpr size_t smem = group_cta_smem_bytes<W, K, KC>();
  uint32_t grid = 0;
  NGIA_TRY(persistent_grid(align_group_cta_kernel<W, K, KC>, 32 * W, smem, kFull, &grid));
  if (KC == 8 && !a.dplanes) return NGIA_ERR_STATE;
  align_group_cta_kernel<W, K, KC><<<grid, 32 * W, smem, s>>>(
      KC == 8 ? a.dplanes : a.packed, a.nib, a.inv, a.offs, a.pairs, a.order, a.bounds, cls,
      cursor, a.scores, a.t, a.fm, a.work);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

// A class of (32 lanes, K words) on one block of kCtaWarps warps per pair
// (32 * kCtaWarps lanes, K / kCtaWarps words): the same rows per ring turn and
// a wider span, so the class's binning holds (align_group_cta.cuh).
// Measured on 2,000,000 heavy-tailed protein pairs (autotuned round): one warp
// per pair 9.28 ms, blocks of two warps 9.69 ms, of four 10.46 ms -- the
// shorter chains do not pay for the extra issue slots and barriers, so the
// block-wide form is off by default (NGIA_CTA_WARPS=2 or 4 at build time).
#ifndef NGIA_CTA_WARPS
#define NGIA_CTA_WARPS 0  // 0: the classes run on one warp per pair (align_group.cuh)
#endif
// the first group class (index within the ladder) run block-wide when
// NGIA_CTA_WARPS is set: 6 = the two widest, (32,8) and (32,16); 4 adds
// (32,4) and (32,6).  On the re-laddered classes, same pairs and box: one
// warp per pair 8.05 ms per round (autotuned), blocks of two warps from
// (32,4) on 8.52 ms, from (32,6) on 8.65 ms.
#ifndef NGIA_CTA_FROM
#define NGIA_CTA_FROM 6
#endif
static_assert(NGIA_CTA_FROM >= 4 && NGIA_CTA_FROM <= 7, "block-wide classes are the G = 32 ones");
constexpr int kCtaWarps = NGIA_CTA_WARPS > 0 ? NGIA_CTA_WARPS : 1;
template <int K>
static int launch_group_cta(const RoundArgs &a, int KC, int cls, unsigned int *cursor,
                            cudaStream_t s) {
  static_assert(K % kCtaWarps == 0, "slices of K / kCtaWarps words");
  constexpr int KW = K / kCtaWarps;
  static_assert((32 * kCtaWarps - 1) * KW + 32 * kCtaWarps >= 31 * K + 32, "span");
  return KC <= 8 ? launch_group_cta_k<kCtaWarps, KW, 8>(a, cls, cursor, s)
                 : launch_group_cta_k<kCtaWarps, KW, 16>(a, cls, cursor, s);
}

template <int W>
static int launch_stream(const RoundArgs &a, int K, int cls, unsigned int *cursor,
                         cudaStream_t s) {
  return K == 5   ? launch_stream_k<W, 5>(a, cls, cursor, s)
         : K == 8 ? launch_stream_k<W, 8>(a, cls, cursor, s)
                  : launch_stream_k<W, 16>(a, cls, cursor, s);
}

template <int G, int K>
static int launch_group(const RoundArgs &a, int KC, int cls, unsigned int *cursor,
                        cudaStream_t s) {
  return KC <= 8 ? launch_group_k<G, K, 8>(a, cls, cursor, s)
                 : launch_group_k<G, K, 16>(a, cls, cursor, s);
}

int launch_align_jobs(const uint32_t *packed, const uint64_t *offs, uint32_t *jobs,
                      uint32_t count, uint32_t identity, cudaStream_t s) {
  if (count == 0) return NGIA_OK;
  align_jobs_kernel<<<ceil_div(count, 128u), 128, 0, s>>>(
      packed, offs, jobs, count, identity_threshold(identity), round_mode());
  NGIA_LAUNCHED();
  return NGIA_OK;
}

int launch_align_jobs_dev_count(const uint32_t *packed, const uint64_t *offs,
                                uint32_t *jobs, const uint32_t *d_count,
                                uint32_t max_count, uint32_t identity,
                                cudaStream_t s) {
  if (max_count == 0) return NGIA_OK;
  const uint32_t blocks = ceil_div(max_count, 128u);
  align_jobs_dev_count_kernel<<<blocks, 128, 0, s>>>(
      packed, offs, jobs, d_count, identity_threshold(identity), round_mode());
  NGIA_LAUNCHED();
  return NGIA_OK;
}

int launch_align_class(int cls, const uint32_t *packed, const uint32_t *nib,
                       const Alphabet &ab, const uint64_t *offs, const uint2 *pairs,
                       const uint32_t *order, const uint32_t *bounds, uint32_t *scores,
                       uint32_t identity, unsigned long long *work, unsigned int *cursor,
                       cudaStream_t s) {
  const RoundArgs a{packed, nib, ab.inv, ab.dplanes, offs, pairs, order, bounds, scores,
                    identity_threshold(identity), round_mode(), work};
  switch (cls) {
#define NGIA_STREAM_CASE(C) \
  case C: return launch_stream<class_width(C)>(a, ab.K, cls, cursor, s);
    NGIA_STREAM_CASE(0)
    NGIA_STREAM_CASE(1)
    NGIA_STREAM_CASE(2)
    NGIA_STREAM_CASE(3)
    NGIA_STREAM_CASE(4)
    NGIA_STREAM_CASE(5)
    NGIA_STREAM_CASE(6)
    NGIA_STREAM_CASE(7)
    NGIA_STREAM_CASE(8)
    NGIA_STREAM_CASE(9)
    NGIA_STREAM_CASE(10)
#undef NGIA_STREAM_CASE
#define NGIA_GROUP_CASE(C) \
  case C: return launch_group<group_shape(C).G, group_shape(C).K>(a, ab.K, cls, cursor, s);
    NGIA_GROUP_CASE(kFirstGroupClass)
    NGIA_GROUP_CASE(kFirstGroupClass + 1)
    NGIA_GROUP_CASE(kFirstGroupClass + 2)
    NGIA_GROUP_CASE(kFirstGroupClass + 3)
#undef NGIA_GROUP_CASE
    // the G = 32 classes, block-wide from NGIA_CTA_FROM on when NGIA_CTA_WARPS is set
#define NGIA_WIDE_CASE(I)                                                                   \
  case kFirstGroupClass + I:                                                                \
    static_assert(group_shape(kFirstGroupClass + I).G == 32, "a G = 32 class");             \
    return NGIA_CTA_WARPS && I >= NGIA_CTA_FROM                                              \
               ? launch_group_cta<group_shape(kFirstGroupClass + I).K>(a, ab.K, cls, cursor, s) \
               : launch_group<32, group_shape(kFirstGroupClass + I).K>(a, ab.K, cls, cursor, s);
    NGIA_WIDE_CASE(4)
    NGIA_WIDE_CASE(5)
    NGIA_WIDE_CASE(6)
    NGIA_WIDE_CASE(7)
#undef NGIA_WIDE_CASE
    static_assert(kNumGroupClasses == 8, "the ladder's cases above");
    case kGeneralClass: {
      uint32_t grid = 0;
      NGIA_TRY(persistent_grid(align_general_kernel, 128, 0, kFull, &grid));
      align_general_kernel<<<grid, 128, 0, s>>>(packed, offs, pairs, order, bounds, cls, scores,
                                                a.t, a.fm, work);
      NGIA_LAUNCHED();
      return NGIA_OK;
    }
    default: return NGIA_ERR_ARG;
  }
}

}  // namespace ngia

extern "C" int ngia_align_pairs(const uint32_t *d_packed, const uint64_t *d_rec_offsets,
                                uint32_t *d_jobs, uint32_t count, uint32_t identity,
                                void *stream) {
  if (identity < 1 || identity > 99) return NGIA_ERR_ARG;
  if (count == 0) return NGIA_OK;
  if (!d_packed || !d_rec_offsets || !d_jobs) return NGIA_ERR_ARG;
  return ngia::launch_align_jobs(d_packed, d_rec_offsets, d_jobs, count, identity,
                                 ngia::as_stream(stream));
}
