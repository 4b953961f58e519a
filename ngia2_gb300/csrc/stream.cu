// stream.cu -- the graph build of a database larger than device memory
// (ngia_stream_graph).  Only the records are streamed: everything that grows
// with the record count but not with the residues (signatures, rep rows,
// lengths, offsets, pairs, scores) stays on the device.
//
// Pass 1, sketch: record chunks (contiguous runs of records, at most
// chunk_words words) are copied host -> pinned staging (CPU) -> device
// (double-buffered: chunk k+1 is staged and copied while chunk k is
// converted to nibble codes and sketched); the first `bands` signature rows
// of each chunk go into the device-wide signature rows, and the residue
// codes present are collected for the aligner's alphabet.
// Then the device path as for a resident database: bucketing of `bands`
// rows, candidates (distinct pairs grouped by target, the reference's length
// filter).
// Pass 2, align: pairs are keyed by (chunk of rep, chunk of target) -- rep
// precedes target, so rep's chunk <= target's -- and sorted by that key.  For
// each outer chunk a (resident in slot 0), the inner chunks b = a, a+1, ... are
// streamed through slots 1 and 2 (b+1 is copied while the block (a, b) is
// aligned); a block's pairs are renumbered into a two-chunk index space
// (a's records, then b's) and aligned by one batched round.  Scores go back to
// the pairs' own positions, so the emission (sorted unique edges) is the
// resident path's.
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "ctx.cuh"

namespace ngia {

// Rebases the offsets and copies the lengths of records [first, first + cnt)
// for a chunk held at word `slot_base` of the region (its first record
// starting at global word `word_first`), at entries [at, at + cnt).
__global__ void __launch_bounds__(256)
region_table_kernel(const uint64_t *__restrict__ offs, const uint32_t *__restrict__ lens,
                    uint32_t first, uint32_t cnt, uint64_t word_first, uint64_t slot_base,
                    uint32_t at, uint64_t *__restrict__ r_offs, uint32_t *__restrict__ r_lens) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  r_offs[at + k] = slot_base + (offs[first + k] - word_first);
  r_lens[at + k] = lens[first + k];
}

// Block key of every pair: chunk(rep) * chunks + chunk(tar).  chunk_first:
// first record of each chunk (ascending), chunks entries.
__global__ void __launch_bounds__(256)
block_key_kernel(const uint2 *__restrict__ pairs, uint32_t m,
                 const uint32_t *__restrict__ chunk_first, uint32_t chunks,
                 uint32_t *__restrict__ keys) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= m) return;
  const uint2 pr = pairs[p];
  auto chunk_of = [&](uint32_t i) {  // last chunk whose first record <= i
    uint32_t lo = 0, hi = chunks;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (chunk_first[mid] <= i) lo = mid;
      else hi = mid;
    }
    return lo;
  };
  keys[p] = chunk_of(pr.x) * chunks + chunk_of(pr.y);
}

// A block's pairs in the region's numbering: records of chunk a are
// 0..na-1, those of chunk b follow (for a == b, b's are a's).
__global__ void __launch_bounds__(256)
block_pairs_kernel(const uint2 *__restrict__ pairs, const uint32_t *__restrict__ order,
                   uint32_t begin, uint32_t cnt, uint32_t first_a, uint32_t na,
                   uint32_t first_b, int same, uint2 *__restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const uint2 pr = pairs[order[begin + k]];
  const uint32_t x = pr.x - first_a;  // the rep is in chunk a
  const uint32_t y = same ? pr.y - first_a : na + (pr.y - first_b);
  out[k] = make_uint2(x, y);
}

__global__ void __launch_bounds__(256)
scatter_block_scores_kernel(const uint32_t *__restrict__ order, uint32_t begin, uint32_t cnt,
                            const uint32_t *__restrict__ block_scores,
                            uint32_t *__restrict__ scores) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < cnt) scores[order[begin + k]] = block_scores[k];
}

using SClock = std::chrono::steady_clock;
static double since_ms(SClock::time_point t) {
  return std::chrono::duration<double, std::milli>(SClock::now() - t).count();
}

struct Chunk {
  uint32_t first, count;      // records
  uint64_t word_first, words;  // word span in the host array
};

// Host copy into pinned staging on several threads: one thread's memcpy
// moves ~10-15 GB/s, well below what the host-to-device link takes.
static void parallel_copy(void *dst, const void *src, size_t bytes) {
  const unsigned hw = std::thread::hardware_concurrency();
  const size_t parts = bytes < (8u << 20) ? 1 : (hw > 1 ? (hw < 16 ? hw : 16) : 1);
  if (parts == 1) {
    std::memcpy(dst, src, bytes);
    return;
  }
  std::vector<std::thread> th;
  const size_t step = (bytes / parts + 4095) & ~size_t(4095);
  for (size_t k = 0; k < parts; ++k) {
    const size_t b = k * step;
    if (b >= bytes) break;
    const size_t e = b + step < bytes ? b + step : bytes;
    th.emplace_back([=] {
      std::memcpy(static_cast<char *>(dst) + b, static_cast<const char *>(src) + b, e - b);
    });
  }
  for (auto &t : th) t.join();
}

// page-locked host memory the device can copy from directly, over the whole
// of [p, p + bytes)
static bool host_pinned(const void *p, size_t bytes) {
  const char *b = static_cast<const char *>(p);
  for (const char *q : {b, b + (bytes ? bytes - 1 : 0)}) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
      (void)cudaGetLastError();
      return false;
    }
    if (a.type != cudaMemoryTypeHost) return false;
  }
  return true;
}

// Pinned double-buffered staging of chunks into the device region's slots.
// stage() copies a chunk's words into one of two pinned buffers (CPU) once
// that buffer's previous copy has reached the device, then issues the
// host-to-device copy on its own stream after the compute stream has
// finished with the destination slot (slot_done[slot], recorded by the
// user after the slot's last reader); the returned event marks the data on
// the device.  When the caller's records are themselves page-locked and span
// at most kDirectMaxBytes, the copy reads them in place and the host copy is
// skipped.  Measured on a GB300 host: 1.09 GB of page-locked records went
// over at 132 GB/s in place against 62 GB/s through the staging buffers,
// but 10.9 GB at 38-60 GB/s in place against 91 GB/s staged (the in-place
// copies walk the whole region's pages; the staging buffers stay small).
constexpr uint64_t kDirectMaxBytes = 4ull << 30;

struct Stager {
  static constexpr int kSlots = 3;
  const uint32_t *h_packed = nullptr;
  bool direct = false;  // the caller's records are page-locked: copied from in place
  uint32_t *pinned[2] = {};
  cudaEvent_t copied_ev[2] = {}, slot_done[kSlots] = {};
  cudaStream_t copy = nullptr;
  int next = 0;
  uint64_t bytes = 0;
  int init(const uint32_t *packed, uint64_t words, uint64_t chunk_words) {
    h_packed = packed;
    direct = words * 4 <= kDirectMaxBytes && host_pinned(packed, words * 4);
    for (int k = 0; k < 2; ++k) {
      if (!direct) NGIA_CUDA(cudaMallocHost(&pinned[k], chunk_words * 4));
      NGIA_CUDA(cudaEventCreateWithFlags(&copied_ev[k], cudaEventDisableTiming));
    }
    for (int k = 0; k < kSlots; ++k)
      NGIA_CUDA(cudaEventCreateWithFlags(&slot_done[k], cudaEventDisableTiming));
    NGIA_CUDA(cudaStreamCreateWithFlags(&copy, cudaStreamNonBlocking));
    return NGIA_OK;
  }
  int stage(const Chunk &c, int slot, uint32_t *dst, cudaEvent_t *copied) {
    const int b = next;
    next ^= 1;
    const uint32_t *src = h_packed + c.word_first;
    if (!direct) {
      NGIA_CUDA(cudaEventSynchronize(copied_ev[b]));  // the pinned buffer's last copy is done
      parallel_copy(pinned[b], src, c.words * 4);
      src = pinned[b];
    }
    NGIA_CUDA(cudaStreamWaitEvent(copy, slot_done[slot], 0));
    NGIA_CUDA(cudaMemcpyAsync(dst, src, c.words * 4, cudaMemcpyHostToDevice, copy));
    NGIA_CUDA(cudaEventRecord(copied_ev[b], copy));
    bytes += c.words * 4;
    *copied = copied_ev[b];
    return NGIA_OK;
  }
  // the compute stream has finished reading `slot` once it passes this point
  int slot_free(int slot, cudaStream_t user) {
    NGIA_CUDA(cudaEventRecord(slot_done[slot], user));
    return NGIA_OK;
  }
  void destroy() {
    if (copy) cudaStreamSynchronize(copy);
    for (int k = 0; k < 2; ++k) {
      if (pinned[k]) cudaFreeHost(pinned[k]);
      if (copied_ev[k]) cudaEventDestroy(copied_ev[k]);
    }
    for (int k = 0; k < kSlots; ++k)
      if (slot_done[k]) cudaEventDestroy(slot_done[k]);
    if (copy) cudaStreamDestroy(copy);
  }
};

// Adds one round's computed blocks and band cells to running totals.
__global__ void accumulate_kernel(const Counters *__restrict__ rc,
                                  unsigned long long *__restrict__ acc) {
  acc[0] += rc->work;
  acc[1] += rc->cells;
}

struct StreamState {
  DevBuf region_packed, region_nib, region_dplanes, r_offs, r_lens;
  DevBuf offs, lens, sigs, sig_tmp, rep, scratch, ucount, uoff, counters, pairs, scores,
      keys, keys_sorted, order, block_pairs, block_scores, chunk_first, presence, emit_tmp,
      edges;
  Round round;
  Stager stager;
  cudaStream_t s = nullptr;
  void destroy() {
    DevBuf *bufs[] = {&region_packed, &region_nib, &region_dplanes, &r_offs, &r_lens,
                      &offs,          &lens,       &sigs,         &sig_tmp, &rep,
                      &scratch,       &ucount,     &uoff,         &counters, &pairs,
                      &scores,        &keys,       &keys_sorted,  &order,   &block_pairs,
                      &block_scores,  &chunk_first, &presence,    &emit_tmp, &edges};
    if (s) cudaStreamSynchronize(s);
    stager.destroy();
    round.destroy();
    for (DevBuf *b : bufs) b->release();
    if (s) cudaStreamDestroy(s);
  }
};

static int stream_graph(StreamState &S, const uint32_t *h_packed, uint64_t words,
                        const uint64_t *h_offs, const uint32_t *h_lens, uint32_t n,
                        uint32_t identity, uint32_t bands, uint64_t chunk_bytes,
                        ngia_edge *h_edges, uint64_t cap, uint64_t *n_edges,
                        ngia_stream_stats *st) {
  const auto t_all = SClock::now();
  // ---- chunks: contiguous runs of records of at most chunk_words words
  // (three chunk slots of planes, nibble codes -- the recoded ones in pass 2 --
  // and code planes in the budget)
  const uint64_t chunk_words = chunk_bytes / (3ull * 4 * 3);
  std::vector<Chunk> chunks;
  for (uint32_t i = 0; i < n; ++i) {
    const uint64_t w = 1 + 4ull * ((h_lens[i] + 31) / 32);
    if (h_lens[i] > NGIA_MAX_READ || h_offs[i] + w > words) return NGIA_ERR_ARG;
    if (i > 0 && h_offs[i] < h_offs[i - 1] + 1 + 4ull * ((h_lens[i - 1] + 31) / 32))
      return NGIA_ERR_ARG;  // records in index order, not overlapping
    if (chunks.empty() || h_offs[i] + w - chunks.back().word_first > chunk_words) {
      if (w > chunk_words) return NGIA_ERR_ARG;  // a record larger than a chunk
      chunks.push_back(Chunk{i, 0, h_offs[i], 0});
    }
    Chunk &c = chunks.back();
    c.count += 1;
    c.words = h_offs[i] + w - c.word_first;
  }
  const uint32_t C = (uint32_t)chunks.size();
  if ((uint64_t)C * C > 0xFFFFFFFFull) return NGIA_ERR_ARG;
  uint32_t max_recs = 0;
  for (const Chunk &c : chunks) max_recs = c.count > max_recs ? c.count : max_recs;

  NGIA_CUDA(cudaStreamCreateWithFlags(&S.s, cudaStreamNonBlocking));
  cudaStream_t s = S.s;
  NGIA_TRY(S.round.init(s));
  NGIA_TRY(S.stager.init(h_packed, words, chunk_words));
  NGIA_TRY(S.region_packed.reserve(3 * chunk_words * 4));
  NGIA_TRY(S.region_nib.reserve(3 * chunk_words * 4));
  NGIA_TRY(S.r_offs.reserve(2ull * max_recs * 8));
  NGIA_TRY(S.r_lens.reserve(2ull * max_recs * 4));
  NGIA_TRY(S.offs.reserve((size_t)n * 8));
  NGIA_TRY(S.lens.reserve((size_t)n * 4));
  NGIA_TRY(S.sigs.reserve((size_t)bands * n * 4));
  NGIA_TRY(S.sig_tmp.reserve((size_t)kBands * max_recs * 4));
  NGIA_TRY(S.presence.reserve((size_t)C * 4 + 32));  // one word per chunk, then totals
  unsigned long long *acc =
      reinterpret_cast<unsigned long long *>(S.presence.as<uint32_t>() + ((C + 1) & ~1u));
  NGIA_TRY(S.counters.reserve(sizeof(Counters)));
  NGIA_CUDA(cudaMemcpyAsync(S.offs.p, h_offs, (size_t)n * 8, cudaMemcpyHostToDevice, s));
  NGIA_CUDA(cudaMemcpyAsync(S.lens.p, h_lens, (size_t)n * 4, cudaMemcpyHostToDevice, s));
  std::vector<uint32_t> firsts(C);
  for (uint32_t k = 0; k < C; ++k) firsts[k] = chunks[k].first;
  NGIA_TRY(S.chunk_first.reserve((size_t)C * 4));
  NGIA_CUDA(cudaMemcpyAsync(S.chunk_first.p, firsts.data(), (size_t)C * 4,
                            cudaMemcpyHostToDevice, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  uint32_t *rp = S.region_packed.as<uint32_t>(), *rn = S.region_nib.as<uint32_t>();
  uint64_t *roffs = S.r_offs.as<uint64_t>();
  uint32_t *rlens = S.r_lens.as<uint32_t>();

  // Loads chunk k into region slot `slot` (planes, and the nibble codes; once
  // the alphabet is known to be dense (pass 2) the recoded codes in their place
  // and the code planes) with its record table at entries [at, at + count);
  // the work is ordered on s.
  uint64_t map = 0;
  bool dense = false;
  auto load_chunk = [&](uint32_t k, int slot, uint32_t at, uint32_t *presence) -> int {
    const Chunk &c = chunks[k];
    const uint64_t base = (uint64_t)slot * chunk_words;
    cudaEvent_t copied;
    NGIA_TRY(S.stager.stage(c, slot, rp + base, &copied));
    NGIA_CUDA(cudaStreamWaitEvent(s, copied, 0));
    region_table_kernel<<<ceil_div(c.count, 256u), 256, 0, s>>>(
        S.offs.as<uint64_t>(), S.lens.as<uint32_t>(), c.first, c.count, c.word_first, base, at,
        roffs, rlens);
    NGIA_LAUNCHED();
    if (dense)
      NGIA_TRY(launch_dense_layouts(rp, roffs + at, c.count, map, rn,
                                    S.region_dplanes.as<uint32_t>(), s));
    else
      NGIA_TRY(launch_nibbles(rp, roffs + at, rlens + at, c.count, base + chunk_words, rn,
                              presence, s));
    return NGIA_OK;
  };

  // ---- pass 1: sketch, chunk by chunk (slots 0 and 1 alternate)
  auto t0 = SClock::now();
  uint32_t present = 0;
  for (uint32_t k = 0; k < C; ++k) {
    const int slot = (int)(k & 1u);
    NGIA_TRY(load_chunk(k, slot, 0, S.presence.as<uint32_t>() + k));
    NGIA_TRY(launch_sketch_nibbles(rn, roffs, chunks[k].count, S.sig_tmp.as<uint32_t>(), s));
    NGIA_CUDA(cudaMemcpy2DAsync(S.sigs.as<uint32_t>() + chunks[k].first, (size_t)n * 4,
                                S.sig_tmp.p, (size_t)chunks[k].count * 4,
                                (size_t)chunks[k].count * 4, bands, cudaMemcpyDeviceToDevice,
                                s));
    NGIA_TRY(S.stager.slot_free(slot, s));
  }
  {  // residue codes present in any chunk
    std::vector<uint32_t> pk(C);
    NGIA_CUDA(cudaMemcpyAsync(pk.data(), S.presence.p, (size_t)C * 4, cudaMemcpyDeviceToHost,
                              s));
    NGIA_CUDA(cudaStreamSynchronize(s));
    for (uint32_t v : pk) present |= v;
  }
  if (present & kBadRecord) return NGIA_ERR_FORMAT;  // a length word not the read length
  const double ms_sketch = since_ms(t0);
  const uint64_t bytes_sketch = S.stager.bytes;

  // ---- the device path: buckets, candidates
  t0 = SClock::now();
  NGIA_TRY(S.rep.reserve((size_t)bands * n * 4));
  NGIA_TRY(S.scratch.reserve(bucket_scratch_bytes(n, bands)));
  NGIA_TRY(bucket(S.sigs.as<uint32_t>(), n, bands, S.rep.as<uint32_t>(), S.scratch.p, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  const double ms_bucket = since_ms(t0);
  t0 = SClock::now();
  Counters *dc = S.counters.as<Counters>();
  NGIA_CUDA(cudaMemsetAsync(dc, 0, sizeof(Counters), s));
  NGIA_TRY(S.ucount.reserve((size_t)n * 4));
  NGIA_TRY(S.uoff.reserve((size_t)n * 8));
  NGIA_TRY(collect_count(S.rep.as<uint32_t>(), S.lens.as<uint32_t>(), n, bands, identity,
                         S.ucount.as<uint32_t>(), &dc->cand_total, s));
  NGIA_TRY(S.scratch.reserve(scan_scratch_bytes(n)));
  NGIA_TRY(exclusive_scan_u64(S.ucount.as<uint32_t>(), S.uoff.as<uint64_t>(), n,
                              &dc->unique_total, S.scratch.as<uint64_t>(), s));
  Counters hc;
  NGIA_CUDA(cudaMemcpyAsync(&hc, dc, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  if (hc.unique_total > 0xFFFFFFFFull) return NGIA_ERR_NOMEM;
  const uint32_t m = (uint32_t)hc.unique_total;
  const size_t mm = m ? m : 1;
  NGIA_TRY(S.pairs.reserve(mm * 8));
  NGIA_TRY(S.scores.reserve(mm * 4));
  NGIA_TRY(collect_write(S.rep.as<uint32_t>(), S.lens.as<uint32_t>(), n, bands, identity,
                         S.uoff.as<uint64_t>(), S.pairs.as<uint2>(), s));
  // block keys and the block order of the pairs
  NGIA_TRY(S.keys.reserve(mm * 4));
  NGIA_TRY(S.keys_sorted.reserve(mm * 4));
  NGIA_TRY(S.order.reserve(mm * 4));
  NGIA_TRY(S.scratch.reserve(radix_sort_scratch_bytes((uint32_t)mm, 1)));
  std::vector<uint32_t> block_begin((size_t)C * C + 1, 0);
  if (m) {
    block_key_kernel<<<ceil_div(m, 256u), 256, 0, s>>>(S.pairs.as<uint2>(), m,
                                                        S.chunk_first.as<uint32_t>(), C,
                                                        S.keys.as<uint32_t>());
    NGIA_LAUNCHED();
    const int kbits = bits_for((uint32_t)((uint64_t)C * C - 1));
    NGIA_TRY(radix_sort_pairs(S.keys.as<uint32_t>(), nullptr, S.keys_sorted.as<uint32_t>(),
                              S.order.as<uint32_t>(), m, 1, 0, kbits > 0 ? kbits : 1,
                              S.scratch.p, s));
    std::vector<uint32_t> ks(m);  // block boundaries from the sorted keys
    NGIA_CUDA(cudaMemcpyAsync(ks.data(), S.keys_sorted.p, (size_t)m * 4, cudaMemcpyDeviceToHost,
                              s));
    NGIA_CUDA(cudaStreamSynchronize(s));
    for (uint32_t k = 0; k < m; ++k) ++block_begin[ks[k] + 1];
    for (size_t b = 0; b < (size_t)C * C; ++b) block_begin[b + 1] += block_begin[b];
  }
  const double ms_pairs = since_ms(t0);

  // ---- pass 2: align, block by block
  t0 = SClock::now();
  S.stager.bytes = 0;
  const uint32_t codes = (uint32_t)__builtin_popcount(present & ~1u);
  Alphabet ab{16, 0xFEDCBA9876543210ull};
  if (codes <= 7) {  // the dense recoding of the resident path
    uint64_t inv = 0;
    int next = 1;
    for (int code = 1; code < 16; ++code) {
      if (!((present >> code) & 1u)) continue;
      map |= (uint64_t)next << (4 * code);
      inv |= (uint64_t)code << (4 * next);
      ++next;
    }
    dense = true;
    NGIA_TRY(S.region_dplanes.reserve(3 * chunk_words * 4));
    ab = Alphabet{next <= 5 ? 5 : 8, inv, S.region_dplanes.as<uint32_t>()};
  }
  uint32_t max_block = 0;
  for (size_t b = 0; b < (size_t)C * C; ++b) {
    const uint32_t cnt = block_begin[b + 1] - block_begin[b];
    max_block = cnt > max_block ? cnt : max_block;
  }
  const size_t mb = max_block ? max_block : 1;
  NGIA_TRY(S.block_pairs.reserve(mb * 8));
  NGIA_TRY(S.block_scores.reserve(mb * 4));
  NGIA_TRY(S.round.reserve(max_block));
  NGIA_CUDA(cudaMemsetAsync(S.scores.p, 0, mm * 4, s));
  const DbView view{rp, rn, ab, roffs, rlens};
  NGIA_CUDA(cudaMemsetAsync(acc, 0, 16, s));
  uint64_t loads = 0;
  int inner = 1;  // slot of the current inner chunk (1 and 2 alternate)
  for (uint32_t a = 0; a < C; ++a) {
    bool a_loaded = false;
    for (uint32_t b = a; b < C; ++b) {
      const size_t blk = (size_t)a * C + b;
      const uint32_t beg = block_begin[blk], cnt = block_begin[blk + 1] - beg;
      if (cnt == 0) continue;
      if (!a_loaded) {
        NGIA_TRY(load_chunk(a, 0, 0, S.presence.as<uint32_t>()));
        a_loaded = true;
        ++loads;
      }
      const bool same = a == b;
      if (!same) {
        // the other inner slot: its copy overlaps the block still using this one
        inner = inner == 1 ? 2 : 1;
        NGIA_TRY(load_chunk(b, inner, chunks[a].count, S.presence.as<uint32_t>()));
        ++loads;
      }
      block_pairs_kernel<<<ceil_div(cnt, 256u), 256, 0, s>>>(
          S.pairs.as<uint2>(), S.order.as<uint32_t>(), beg, cnt, chunks[a].first,
          chunks[a].count, chunks[b].first, same ? 1 : 0, S.block_pairs.as<uint2>());
      NGIA_LAUNCHED();
      NGIA_TRY(S.round.enqueue(view, S.block_pairs.as<uint2>(), cnt, identity,
                               S.block_scores.as<uint32_t>(), nullptr));
      scatter_block_scores_kernel<<<ceil_div(cnt, 256u), 256, 0, s>>>(
          S.order.as<uint32_t>(), beg, cnt, S.block_scores.as<uint32_t>(),
          S.scores.as<uint32_t>());
      NGIA_LAUNCHED();
      accumulate_kernel<<<1, 1, 0, s>>>(S.round.counters(), acc);  // before the next round
      NGIA_LAUNCHED();
      NGIA_TRY(S.stager.slot_free(0, s));
      if (!same) NGIA_TRY(S.stager.slot_free(inner, s));
    }
  }
  unsigned long long totals[2] = {0, 0};
  NGIA_CUDA(cudaMemcpyAsync(totals, acc, 16, cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  const unsigned long long work = totals[0], cells = totals[1];
  const double ms_align = since_ms(t0);
  const uint64_t bytes_align = S.stager.bytes;

  // ---- emission: sorted unique edges, as the resident path
  t0 = SClock::now();
  NGIA_TRY(S.emit_tmp.reserve(emit_scratch_bytes(m, n)));
  NGIA_TRY(S.edges.reserve(mm * sizeof(ngia_edge)));
  uint64_t ne = 0;
  NGIA_TRY(emit_sorted(S.pairs.as<uint2>(), S.scores.as<uint32_t>(), m, n,
                       S.edges.as<ngia_edge>(), &ne, S.emit_tmp.p, s));
  if (ne > cap) return NGIA_ERR_NOMEM;
  if (ne) NGIA_CUDA(cudaMemcpyAsync(h_edges, S.edges.p, ne * sizeof(ngia_edge),
                                    cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  *n_edges = ne;
  if (st) {
    st->chunks = C;
    st->chunk_loads = C + loads;
    st->bytes_h2d_sketch = bytes_sketch;
    st->bytes_h2d_align = bytes_align;
    st->candidate_pairs = hc.cand_total;
    st->unique_pairs = m;
    st->aligned_cells = cells;
    st->computed_cells = work * 1024ull;
    st->edges = ne;
    st->ms_sketch = ms_sketch;
    st->ms_bucket = ms_bucket;
    st->ms_pairs = ms_pairs;
    st->ms_align = ms_align;
    st->ms_emit = since_ms(t0);
    st->ms_total = since_ms(t_all);
  }
  return NGIA_OK;
}

}  // namespace ngia

extern "C" int ngia_stream_graph(const uint32_t *h_packed, uint64_t words,
                                 const uint64_t *h_offs, const uint32_t *h_lens, uint32_t n,
                                 uint32_t identity, uint32_t bands, uint64_t chunk_bytes,
                                 ngia_edge *h_edges, uint64_t cap, uint64_t *n_edges,
                                 ngia_stream_stats *stats) {
  if (!h_packed || !h_offs || !h_lens || !n_edges || n == 0 || (cap && !h_edges))
    return NGIA_ERR_ARG;
  if (identity < 1 || identity > 99 || bands < 1 || bands > NGIA_BANDS) return NGIA_ERR_ARG;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  *n_edges = 0;
  ngia::StreamState S;
  const int rc = ngia::stream_graph(S, h_packed, words, h_offs, h_lens, n, identity, bands,
                                    chunk_bytes, h_edges, cap, n_edges, stats);
  S.destroy();
  return rc;
}
