// sketch.cu -- stage (a): 64 minhash signatures per packed record.
//
// Restates the signing loop of MakeDB::packData (src/makedb.hpp:224-248):
//   k-mer  = the last 8 residue codes as one 32-bit word, newest code in the
//            low nibble (codes before position 0 are 0);
//   signed positions: 7..L-1, or only L-1 when L < 8; none when L = 0;
//   band k = min over signed positions of H(kmer ^ (k*0x9e3779b1 + 0x85ebca6b))
//   with H Wang's 32-bit integer hash followed by two extra xor-shift-multiply
//   rounds (the steps below), minimum 0xFFFFFFFF when nothing is signed.
//
// Mapping: one warp per record; each lane signs a contiguous run of the
// positions and keeps all 64 running minima in registers (64 independent
// hash chains per position), then one redux.sync min per band combines the
// lanes.  Records are in length-descending index order, so the longest are
// scheduled first.
//
// The work is integer-bound: 64 hashes of 13 integer instructions per
// position against half a byte read.  On this GPU the logic/shift pipe and
// the integer multiply-add pipe draw on the same integer issue budget, and a
// multiply-high costs two of its slots, so the shifts stay shifts.
#include "kernels.cuh"

namespace ngia {

// First xor-shift of the hash with the band seed folded in:
//   x = kmer ^ seed;  x = (x ^ 61) ^ (x >> 16)
//     = (kmer ^ (kmer >> 16)) ^ (seed ^ 61 ^ (seed >> 16))
__host__ __device__ constexpr uint32_t band_seed_fold(uint32_t band) {
  return (band * 0x9e3779b1u + 0x85ebca6bu) ^ 61u ^
         ((band * 0x9e3779b1u + 0x85ebca6bu) >> 16);
}

__device__ __forceinline__ uint32_t band_hash_tail(uint32_t x) {
  x = x * 9u;  // x + (x << 3)
  x ^= x >> 4;
  x *= 0x27d4eb2du;
  x ^= x >> 15;
  x = (x ^ (x >> 8)) * 0x9e3779b1u;
  x ^= x >> 14;
  return x;
}

// k-mers from the bit planes of a packed record (ABI entry point).
struct PlaneKmers {
  const uint32_t *rec;
  __device__ static PlaneKmers make(const uint32_t *r) {
    PlaneKmers k;
    k.rec = r;
    return k;
  }
  uint32_t block = 0xFFFFFFFFu;
  uint32_t p0 = 0, p1 = 0, p2 = 0, p3 = 0;
  uint32_t kmer = 0;
  __device__ __forceinline__ uint32_t code(uint32_t pos) {
    const uint32_t blk = pos >> 5;
    if (blk != block) {
      const uint32_t *b = rec + 1 + 4 * blk;
      p0 = __ldg(b);
      p1 = __ldg(b + 1);
      p2 = __ldg(b + 2);
      p3 = __ldg(b + 3);
      block = blk;
    }
    const uint32_t s = pos & 31u;
    return ((p0 >> s) & 1u) | (((p1 >> s) & 1u) << 1) | (((p2 >> s) & 1u) << 2) |
           (((p3 >> s) & 1u) << 3);
  }
  __device__ __forceinline__ void start(uint32_t pb) {
    kmer = 0;
    for (uint32_t q = pb >= 7 ? pb - 7 : 0; q < pb; ++q) kmer = (kmer << 4) | code(q);
  }
  __device__ __forceinline__ uint32_t at(uint32_t p) {  // positions in increasing order
    kmer = (kmer << 4) | code(p);
    return kmer;
  }
};

// k-mers from the nibble layout (word k holds positions 8k..8k+7, first in the
// high nibble): the k-mer ending at p is the 32-bit window of the stream
// starting at position p - 7, one funnel shift.
struct NibbleKmers {
  const uint32_t *nib;  // the record's first code word
  __device__ static NibbleKmers make(const uint32_t *r) { return NibbleKmers{r + 1}; }
  __device__ __forceinline__ void start(uint32_t) {}
  __device__ __forceinline__ uint32_t at(uint32_t p) {
    if (p < 7) return __ldg(nib) >> (28 - 4 * p);  // short record: codes 0..p
    const uint32_t s = p - 7, k = s >> 3, r = s & 7u;
    const uint32_t hi = __ldg(nib + k);
    return r ? __funnelshift_l(__ldg(nib + k + 1), hi, 4 * r) : hi;
  }
};

template <typename Source>
__global__ void __launch_bounds__(256)
sketch_kernel(const uint32_t *__restrict__ words, const uint64_t *__restrict__ offs,
              uint32_t n, uint32_t *__restrict__ sigs) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const uint32_t *rec = words + offs[i];
    const uint32_t len = __ldg(rec);
    const uint32_t first = len >= 8 ? 7u : (len > 0 ? len - 1 : 0u);
    const uint32_t span = len - first;  // signed positions
    const uint32_t per = (span + 31u) >> 5;
    const uint32_t pb = first + lane * per;
    const uint32_t pe = min(pb + per, len);

    uint32_t mn[kBands];
#pragma unroll
    for (int k = 0; k < kBands; ++k) mn[k] = kFull;

    if (pb < pe) {
      Source src = Source::make(rec);
      src.start(pb);
      for (uint32_t p = pb; p < pe; ++p) {
        const uint32_t kmer = src.at(p);
        const uint32_t y = kmer ^ (kmer >> 16);
#pragma unroll
        for (int k = 0; k < kBands; ++k)
          mn[k] = min(mn[k], band_hash_tail(y ^ band_seed_fold((uint32_t)k)));
      }
    }
    uint32_t lo = kFull, hi = kFull;
#pragma unroll
    for (int k = 0; k < kBands; ++k) {
      const uint32_t r = __reduce_min_sync(kFull, mn[k]);
      if ((uint32_t)(k & 31) == lane) {
        if (k < 32) lo = r;
        else hi = r;
      }
    }
    sigs[(size_t)lane * n + i] = lo;
    sigs[(size_t)(lane + 32) * n + i] = hi;
  }
}

template <typename Source>
static int launch(const uint32_t *words, const uint64_t *offs, uint32_t n, uint32_t *sigs,
                  cudaStream_t s) {
  if (n == 0) return NGIA_OK;
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint32_t want = ceil_div(n, 8u);  // 8 warps per block
  const uint32_t cap = (uint32_t)sms * 16u;
  sketch_kernel<Source><<<want < cap ? want : cap, 256, 0, s>>>(words, offs, n, sigs);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

int launch_sketch(const uint32_t *packed, const uint64_t *offs, uint32_t n, uint32_t *sigs,
                  cudaStream_t s) {
  return launch<PlaneKmers>(packed, offs, n, sigs, s);
}

int launch_sketch_nibbles(const uint32_t *nib, const uint64_t *offs, uint32_t n,
                          uint32_t *sigs, cudaStream_t s) {
  return launch<NibbleKmers>(nib, offs, n, sigs, s);
}

// ---- databases of at most four residue codes: tables of all 8-mers -------------
// With at most four codes (nucleotides) an 8-mer is one of 4^8 = 65,536
// values.  Entry idx of the tables (2 bits per position, the newest in the low
// bits; digit d is aligner code d + 1, i.e. the residue code in nibble d + 1
// of `inv`) stands for the k-mer kmer_of_index(idx), whose hashes are exactly
// those sketch_kernel computes, so the signatures are the same.  Two tables:
//
//  * the ranks: per band, the 65,536 entries in increasing order of that
//    band's hash.  A band's minimum over a record is the hash of the first
//    entry in this order that occurs in the record.  A warp marks the
//    record's 8-mers in a 65,536-bit set in shared memory, then each lane
//    walks the orders of two bands, 8 entries per 16-byte load, until each
//    has met an 8-mer of the record: ~45 bit tests per band for a record of
//    1,500 positions instead of 1,500 hashes per band (the warp waits for its
//    slowest lane, ~3x the mean).  The expected walk grows as
//    65,536 / positions, so
//  * short records (fewer than kRankMinSpan signed positions) take the hash
//    row table: bands [0, kTableBands) of every 8-mer, gathered with 16-byte
//    loads while the other bands are hashed as in sketch_kernel (gathering
//    all 64 is bound by L2 bandwidth, hashing all by the logic pipe).
#ifndef NGIA_SKETCH_TABLE_BANDS
#define NGIA_SKETCH_TABLE_BANDS 24  // multiple of 4
#endif
#ifndef NGIA_SKETCH_RANK_MIN_SPAN
#define NGIA_SKETCH_RANK_MIN_SPAN 512
#endif
constexpr int kTableBands = NGIA_SKETCH_TABLE_BANDS;
static_assert(kTableBands % 4 == 0 && kTableBands <= kBands, "table bands");
constexpr uint32_t kRankMinSpan = NGIA_SKETCH_RANK_MIN_SPAN;
constexpr uint32_t kBitsetWords = kSketchTableEntries / 32;
constexpr uint32_t kRankWarps = 4;  // warps per block, one 8 KB bit set each
constexpr size_t kRowTableBytes = (size_t)kSketchTableEntries * kTableBands * 4;
constexpr size_t kRankBytes = (size_t)kSketchTableEntries * kBands * 2;

__device__ __forceinline__ uint32_t kmer_of_index(uint32_t idx, uint64_t inv) {
  uint32_t kmer = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint32_t d = (idx >> (2 * j)) & 3u;
    kmer |= ((uint32_t)(inv >> (4 * (d + 1))) & 15u) << (4 * j);
  }
  return kmer;
}

__device__ __forceinline__ uint32_t index_hash(uint32_t idx, uint64_t inv, uint32_t band) {
  const uint32_t kmer = kmer_of_index(idx, inv);
  return band_hash_tail((kmer ^ (kmer >> 16)) ^ band_seed_fold(band));
}

// rows[idx * kTableBands + band] for the first kTableBands bands
__global__ void __launch_bounds__(256)
sketch_rows_build_kernel(uint64_t inv, uint32_t *__restrict__ rows) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= kSketchTableEntries * (uint32_t)kTableBands) return;
  rows[t] = index_hash(t / kTableBands, inv, t % kTableBands);
}

// band-major (hash, entry) pairs of all 64 bands, to be sorted per band
__global__ void __launch_bounds__(256)
sketch_keys_build_kernel(uint64_t inv, uint32_t *__restrict__ keys,
                         uint32_t *__restrict__ vals) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= kSketchTableEntries * (uint32_t)kBands) return;
  const uint32_t idx = t % kSketchTableEntries;
  keys[t] = index_hash(idx, inv, t / kSketchTableEntries);
  vals[t] = idx;
}

__global__ void __launch_bounds__(256)
narrow_kernel(const uint32_t *__restrict__ in, uint16_t *__restrict__ out, uint32_t count) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) out[t] = (uint16_t)in[t];
}

// A word of eight 2-bit digits held one per nibble (first position in the
// high nibble) -> the table entry of that 8-mer (the newest digit lowest).
__device__ __forceinline__ uint32_t compress_digits(uint32_t t) {
  t = (t | (t >> 2)) & 0x0F0F0F0Fu;
  t = (t | (t >> 4)) & 0x00FF00FFu;
  return (t | (t >> 8)) & 0x0000FFFFu;
}

// Rolling 8-mer entry over positions [pb, pe) of a record in aligner codes
// (word k holds positions 8k..8k+7, first in the high nibble); f(p, idx).
template <typename F>
__device__ __forceinline__ void for_each_index(const uint32_t *w, uint32_t pb, uint32_t pe,
                                               F &&f) {
  uint32_t idx = 0;
  for (uint32_t q = pb - 7; q < pb; ++q)
    idx = (idx << 2) | (((__ldg(w + (q >> 3)) >> (28 - 4 * (q & 7u))) & 15u) - 1u);
  uint32_t word = __ldg(w + (pb >> 3));
  for (uint32_t p = pb; p < pe; ++p) {
    if ((p & 7u) == 0) word = __ldg(w + (p >> 3));
    idx = ((idx << 2) | (((word >> (28 - 4 * (p & 7u))) & 15u) - 1u)) & 0xFFFFu;
    f(p, idx);
  }
}

// Records with at least kRankMinSpan signed positions: the rank walk.
__global__ void __launch_bounds__(kRankWarps * 32)
sketch_rank_kernel(const uint32_t *__restrict__ dense, const uint64_t *__restrict__ offs,
                   uint32_t n, uint64_t words, uint64_t inv, const uint16_t *__restrict__ ranks,
                   uint32_t *__restrict__ sigs, uint32_t stride) {
  __shared__ __align__(16) uint32_t bitsets[kRankWarps * kBitsetWords];
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t *bits = bitsets + (threadIdx.x >> 5) * kBitsetWords;
  uint4 *bits4 = reinterpret_cast<uint4 *>(bits);
#pragma unroll
  for (uint32_t k = 0; k < kBitsetWords / 128; ++k) bits4[k * 32 + lane] = make_uint4(0, 0, 0, 0);
  __syncwarp();
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const uint64_t o = offs[i];
    if (o >= words) continue;  // outside the layouts (flagged by their kernel)
    const uint32_t len = __ldg(dense + o);
    if (len < 7 + kRankMinSpan) continue;  // short: the row table kernel's
    if (o + 1 + 4ull * ((len + 31u) >> 5) > words) continue;
    // mark the 8-mers: lane l takes code words l, l + 32, ... (coalesced), the
    // entry rolling over the word's 8 positions from the previous word's last
    const uint32_t *w = dense + o + 1;
    const uint32_t words = (len + 7) >> 3;
    for (uint32_t k = lane; k < words; k += 32) {
      uint32_t cur = __ldg(w + k);
      const uint32_t valid = len - 8 * k;  // codes in this word (1..8 in the last)
      if (valid < 8) cur |= 0x11111111u >> (4 * valid);  // padding: any code, never read
      cur -= 0x11111111u;                  // digits 0..3, no borrows
      uint32_t idx = k ? compress_digits(__ldg(w + k - 1) - 0x11111111u) : 0u;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        idx = ((idx << 2) | ((cur >> (28 - 4 * r)) & 3u)) & 0xFFFFu;
        if (8 * k + r >= 7 && (uint32_t)r < valid)
          atomicOr(bits + (idx >> 5), 1u << (idx & 31u));
      }
    }
    __syncwarp();
    // walk: lane l finds the minima of bands l and l + 32 in turn, testing
    // 8 entries of the band's order per 16-byte load, two loads ahead
    uint32_t hit[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint4 *row = reinterpret_cast<const uint4 *>(ranks) +
                         (size_t)(lane + 32 * h) * (kSketchTableEntries / 8);
      uint4 cur = __ldg(row), nxt = __ldg(row + 1);
      uint32_t found = kFull;
      // bounded: the record has an 8-mer, so every band's order meets it
      for (uint32_t step = 0; found == kFull && step < kSketchTableEntries / 8; ++step) {
        const uint4 v = cur;
        cur = nxt;
        nxt = __ldg(row + min(step + 2, kSketchTableEntries / 8 - 1));
        const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
        uint32_t hm = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const uint32_t e = (wv[q >> 1] >> (16 * (q & 1))) & 0xFFFFu;
          hm |= ((bits[e >> 5] >> (e & 31u)) & 1u) << q;
        }
        if (hm) {
          const int q = __ffs(hm) - 1;
          found = (wv[q >> 1] >> (16 * (q & 1))) & 0xFFFFu;
        }
      }
      hit[h] = found;
    }
    __syncwarp();
#pragma unroll
    for (uint32_t k = 0; k < kBitsetWords / 128; ++k)
      bits4[k * 32 + lane] = make_uint4(0, 0, 0, 0);
    const uint32_t lo = index_hash(hit[0], inv, lane);
    const uint32_t hi = index_hash(hit[1], inv, lane + 32);
    __syncwarp();
    sigs[(size_t)lane * stride + i] = lo;
    sigs[(size_t)(lane + 32) * stride + i] = hi;
  }
}

// Records with fewer than kRankMinSpan signed positions: row table + hashing.
// packed: the records' bit planes (residue codes for the hashed bands, and
// records shorter than 8, hashed directly); dense: the same records in
// aligner codes 1..4 (the table's index).
__global__ void __launch_bounds__(256)
sketch_table_kernel(const uint32_t *__restrict__ packed, const uint32_t *__restrict__ dense,
                    const uint64_t *__restrict__ offs, uint32_t n, uint64_t words,
                    const uint4 *__restrict__ table, uint32_t *__restrict__ sigs,
                    uint32_t stride) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const uint64_t o = offs[i];
    if (o >= words) continue;  // outside the layouts (flagged by their kernel)
    const uint32_t len = __ldg(packed + o);
    if (len >= 7 + kRankMinSpan) continue;  // the rank walk's
    if (o + 1 + 4ull * ((len + 31u) >> 5) > words) continue;
    uint32_t mn[kBands];
#pragma unroll
    for (int k = 0; k < kBands; ++k) mn[k] = kFull;
    if (len >= 8) {
      const uint32_t span = len - 7;  // signed positions 7 .. len-1
      const uint32_t per = (span + 31u) >> 5;
      const uint32_t pb = 7 + lane * per;
      const uint32_t pe = min(pb + per, len);
      if (pb < pe) {
        PlaneKmers src = PlaneKmers::make(packed + o);  // rolled along the lane's run
        src.start(pb);
        for_each_index(dense + o + 1, pb, pe, [&](uint32_t p, uint32_t idx) {
          const uint4 *row = table + (size_t)idx * (kTableBands / 4);
          uint4 v[kTableBands / 4];
#pragma unroll
          for (int k = 0; k < kTableBands / 4; ++k) v[k] = __ldg(row + k);
          // the other bands are hashed while the row is on its way
          const uint32_t kmer = src.at(p);
          const uint32_t y = kmer ^ (kmer >> 16);
#pragma unroll
          for (int k = kTableBands; k < kBands; ++k)
            mn[k] = min(mn[k], band_hash_tail(y ^ band_seed_fold((uint32_t)k)));
#pragma unroll
          for (int k = 0; k < kTableBands / 4; ++k) {
            mn[4 * k] = min(mn[4 * k], v[k].x);
            mn[4 * k + 1] = min(mn[4 * k + 1], v[k].y);
            mn[4 * k + 2] = min(mn[4 * k + 2], v[k].z);
            mn[4 * k + 3] = min(mn[4 * k + 3], v[k].w);
          }
        });
      }
    } else if (len > 0 && lane == 0) {  // the one signed position: the whole record
      PlaneKmers src = PlaneKmers::make(packed + o);
      src.start(len - 1);
      const uint32_t kmer = src.at(len - 1);
      const uint32_t y = kmer ^ (kmer >> 16);
#pragma unroll
      for (int k = 0; k < kBands; ++k) mn[k] = band_hash_tail(y ^ band_seed_fold((uint32_t)k));
    }
    uint32_t lo = kFull, hi = kFull;
#pragma unroll
    for (int k = 0; k < kBands; ++k) {
      const uint32_t r = __reduce_min_sync(kFull, mn[k]);
      if ((uint32_t)(k & 31) == lane) {
        if (k < 32) lo = r;
        else hi = r;
      }
    }
    sigs[(size_t)lane * stride + i] = lo;
    sigs[(size_t)(lane + 32) * stride + i] = hi;
  }
}

size_t sketch_table_bytes() { return kRowTableBytes + kRankBytes; }

int build_sketch_table(uint64_t inv, void *table, cudaStream_t s) {
  uint8_t *base = static_cast<uint8_t *>(table);
  const uint32_t rows = kSketchTableEntries * (uint32_t)kTableBands;
  sketch_rows_build_kernel<<<ceil_div(rows, 256u), 256, 0, s>>>(
      inv, reinterpret_cast<uint32_t *>(base));
  NGIA_LAUNCHED();
  // the ranks: sort (hash, entry) per band, keep the entries as 16 bits
  const uint32_t total = kSketchTableEntries * (uint32_t)kBands;
  const size_t sort_bytes = radix_sort_scratch_bytes(kSketchTableEntries, kBands);
  void *tmp = nullptr;
  NGIA_CUDA(cudaMallocAsync(&tmp, (size_t)total * 16 + sort_bytes, s));
  uint32_t *keys = static_cast<uint32_t *>(tmp), *vals = keys + total;
  uint32_t *keys_out = vals + total, *vals_out = keys_out + total;
  sketch_keys_build_kernel<<<ceil_div(total, 256u), 256, 0, s>>>(inv, keys, vals);
  NGIA_LAUNCHED();
  int rc = radix_sort_pairs(keys, vals, keys_out, vals_out, kSketchTableEntries, kBands, 0,
                            32, vals_out + total, s);
  if (rc == NGIA_OK) {
    narrow_kernel<<<ceil_div(total, 256u), 256, 0, s>>>(
        vals_out, reinterpret_cast<uint16_t *>(base + kRowTableBytes), total);
    NGIA_LAUNCHED();
  }
  NGIA_CUDA(cudaFreeAsync(tmp, s));
  return rc;
}

static int rank_blocks_per_sm() {
  static int cached = 0;
  if (!cached) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, sketch_rank_kernel,
                                                      kRankWarps * 32, 0) != cudaSuccess ||
        b < 1)
      b = 1;
    cached = b;
  }
  return cached;
}

int launch_sketch_table(const uint32_t *packed, const uint32_t *dense, const uint64_t *offs,
                        uint32_t n, uint64_t words, uint64_t inv, const void *table,
                        uint32_t *sigs, uint32_t stride, cudaStream_t s, cudaStream_t side,
                        cudaEvent_t fork, cudaEvent_t join) {
  if (n == 0) return NGIA_OK;
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint8_t *base = static_cast<const uint8_t *>(table);
  // The rank walk's residency is bound by its bit sets (shared memory), which
  // leaves each SM room in threads and registers for one block of the short
  // records' kernel (no shared memory): one block per SM, beside it.
  NGIA_CUDA(cudaEventRecord(fork, s));
  NGIA_CUDA(cudaStreamWaitEvent(side, fork, 0));
  const uint32_t want = ceil_div(n, 8u), cap = (uint32_t)sms;
  sketch_table_kernel<<<want < cap ? want : cap, 256, 0, side>>>(
      packed, dense, offs, n, words, reinterpret_cast<const uint4 *>(base), sigs, stride);
  NGIA_LAUNCHED();
  const uint32_t rank_want = ceil_div(n, kRankWarps);
  const uint32_t rank_cap = (uint32_t)(sms * rank_blocks_per_sm());
  sketch_rank_kernel<<<rank_want < rank_cap ? rank_want : rank_cap, kRankWarps * 32, 0, s>>>(
      dense, offs, n, words, inv, reinterpret_cast<const uint16_t *>(base + kRowTableBytes),
      sigs, stride);
  NGIA_LAUNCHED();
  if (join) {
    NGIA_CUDA(cudaEventRecord(join, side));
    NGIA_CUDA(cudaStreamWaitEvent(s, join, 0));
  }
  return NGIA_OK;
}

}  // namespace ngia

extern "C" int ngia_sketch_table_bands(void) { return ngia::kTableBands; }

extern "C" int ngia_sketch(const uint32_t *d_packed, const uint64_t *d_rec_offsets,
                           uint32_t n, uint32_t *d_sigs, void *stream) {
  if (n == 0) return NGIA_OK;
  if (!d_packed || !d_rec_offsets || !d_sigs) return NGIA_ERR_ARG;
  return ngia::launch_sketch(d_packed, d_rec_offsets, n, d_sigs, ngia::as_stream(stream));
}
