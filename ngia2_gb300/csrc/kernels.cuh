// kernels.cuh -- launchers shared between the translation units of libngia
// (internal header).
#pragma once

#include "align.cuh"

namespace ngia {

// sketch.cu
int launch_sketch(const uint32_t *packed, const uint64_t *offs, uint32_t n,
                  uint32_t *sigs, cudaStream_t s);
int launch_sketch_nibbles(const uint32_t *nib, const uint64_t *offs, uint32_t n,
                          uint32_t *sigs, cudaStream_t s);
// Databases of at most four residue codes (none of them 0): an 8-mer is one of
// kSketchTableEntries values.  build_sketch_table fills sketch_table_bytes()
// of device memory from the aligner codes' inverse map (part of the band
// hashes of every 8-mer, and per band the 8-mers in increasing hash order);
// the sketch then reads the aligner codes (dense).
constexpr uint32_t kSketchTableEntries = 1u << 16;
size_t sketch_table_bytes();
int build_sketch_table(uint64_t inv, void *table, cudaStream_t s);
// Records offs[0..n) (a run of a database's records), signatures at
// sigs[band * stride + i].  The short records' kernel runs on `side` (forked
// from s through `fork`, joined back through `join`; join = null: the caller
// joins later) beside the rank walk on s.  A record whose offset or length
// word puts it past `words` (the layouts' size) is skipped, so the kernels
// stay inside the layouts whatever the offsets hold.
int launch_sketch_table(const uint32_t *packed, const uint32_t *dense, const uint64_t *offs,
                        uint32_t n, uint64_t words, uint64_t inv, const void *table,
                        uint32_t *sigs, uint32_t stride, cudaStream_t s, cudaStream_t side,
                        cudaEvent_t fork, cudaEvent_t join);

// sort.cu
// One-time per-device setup of the sort kernels (attributes); done by the
// first sort, or ahead of a stream capture.
int sort_prepare();
size_t radix_sort_scratch_bytes(uint32_t seg_len, uint32_t segs);
int radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in,
                     uint32_t *keys_out, uint32_t *vals_out, uint32_t seg_len,
                     uint32_t segs, int begin_bit, int end_bit, void *scratch,
                     cudaStream_t s);
size_t scan_scratch_bytes(uint32_t n);
int exclusive_scan_u64(const uint32_t *in, uint64_t *out, uint32_t n,
                       uint64_t *d_total, void *scratch, cudaStream_t s);

// bucket.cu
size_t bucket_scratch_bytes(uint32_t n, uint32_t bands);
int bucket(const uint32_t *sigs, uint32_t n, uint32_t bands, uint32_t *rep,
           void *scratch, cudaStream_t s);

// align.cu
int launch_align_jobs(const uint32_t *packed, const uint64_t *offs, uint32_t *jobs,
                      uint32_t count, uint32_t identity, cudaStream_t s);
int launch_align_jobs_dev_count(const uint32_t *packed, const uint64_t *offs,
                                uint32_t *jobs, const uint32_t *d_count,
                                uint32_t max_count, uint32_t identity,
                                cudaStream_t s);
// Alphabet of the target codes the aligner reads: codes 1..K-1 in use;
// inv packs, per code d < K, the residue code whose match mask d stands for
// (identity when the codes were not recoded).
struct Alphabet {
  int K;         // 5, 8 or 16 table entries per row block (aligner codes 0..K-1)
  uint64_t inv;  // nibble d = residue code of aligner code d
  // K < 16: the records with their bit planes holding the aligner codes
  // (planes 0-2; same layout and offsets as the packed records), from which a
  // row block's table entries are one logic op each
  const uint32_t *dplanes = nullptr;
};
// One width class of the batched aligner: a persistent launch over
// order[bounds[cls], bounds[cls + 1]) (device bounds, from classify).  `cursor`
// (device, zero before the launch) is the class's queue head.
int launch_align_class(int cls, const uint32_t *packed, const uint32_t *nib,
                       const Alphabet &ab, const uint64_t *offs, const uint2 *pairs,
                       const uint32_t *order, const uint32_t *bounds, uint32_t *scores,
                       uint32_t identity, unsigned long long *work, unsigned int *cursor,
                       cudaStream_t s);
// All layouts of records offs[0..n) in one pass under an assumed code map
// (inv: nibble d = residue code of aligner code d, pipelined loads): nibbles,
// recoded nibbles and code planes.  *bad = 1 if a residue has a code outside
// the map or a record is not inside words [w0, w1) (such a record is skipped).
// (A record whose length word is not lens[i] sets *bad too.)
int launch_load_layouts(const uint32_t *packed, const uint64_t *offs, const uint32_t *lens,
                        uint32_t n, uint64_t w0, uint64_t w1, uint64_t words, uint64_t inv,
                        uint32_t *dense_nib, uint32_t *dplanes, uint32_t *bad,
                        cudaStream_t s);
// presence |= the codes seen (cleared first unless accumulate); a record
// outside the region's `words`, or whose length word is not lens[i], is
// skipped and sets kBadRecord.
constexpr uint32_t kBadRecord = 1u << 31;
int launch_nibbles(const uint32_t *packed, const uint64_t *offs, const uint32_t *lens,
                   uint32_t n, uint64_t words, uint32_t *nib, uint32_t *presence, cudaStream_t s,
                   bool accumulate = false);
// Packed records and a code map with new codes 0..7 -> the recoded nibbles
// (residue code c -> map nibble c) and the planes of the new codes
// (Alphabet::dplanes), in one pass.
int launch_dense_layouts(const uint32_t *packed, const uint64_t *offs, uint32_t n,
                         uint64_t map, uint32_t *dense_nib, uint32_t *dplanes,
                         cudaStream_t s);

// pack.cu
// Residue text -> packed records (planes), their nibble layout and the codes
// present (cleared first), in one pass; record i's residues at res + starts[i].
int launch_pack_layout(const uint8_t *res, const uint64_t *starts, const uint32_t *lens,
                       uint32_t n, const uint64_t *offs, uint32_t *packed, uint32_t *nib,
                       uint32_t *presence, cudaStream_t s);

// pairs.cu
// Candidate pairs in one pass (see pairs.cu): pairs[] must hold bands * n;
// *ticket and *unique_total zero before the call, status[] holds
// ceil(n / 32) words (cleared here); *error set if a look-back gave up after
// spin_limit polls of a predecessor's status.
constexpr uint32_t kLookbackSpins = 1u << 22;
int collect_scan(const uint32_t *rep, const uint32_t *lens, uint32_t n, uint32_t bands,
                 uint32_t identity, unsigned int *ticket, unsigned long long *status,
                 unsigned long long *cand_total, uint64_t *unique_total, unsigned int *error,
                 uint2 *pairs, cudaStream_t s, uint32_t spin_limit = kLookbackSpins);
int collect_count(const uint32_t *rep, const uint32_t *lens, uint32_t n, uint32_t bands,
                  uint32_t identity, uint32_t *ucount, unsigned long long *cand_total,
                  cudaStream_t s);
int collect_write(const uint32_t *rep, const uint32_t *lens, uint32_t n, uint32_t bands,
                  uint32_t identity, const uint64_t *offsets, uint2 *pairs,
                  cudaStream_t s);
// Width class sort keys of `count` pairs, per-class counts (added to
// class_count), band cells (added to *cells) and the class bounds of the
// class-major order (bounds[c] = pairs in classes below c; kNumClasses + 1
// entries, written after the counts are complete).
int classify(const uint32_t *lens, const uint2 *pairs, uint32_t count, uint32_t identity,
             const ClassPlan &plan, uint32_t *cls, unsigned int *class_count,
             unsigned long long *cells, uint32_t *bounds, cudaStream_t s);
int bits_for(uint32_t max_value);
// The part-th of `parts` contiguous ranges [h_cut[0], h_cut[1]) of the pairs,
// cut so that each holds about 1/parts of their band blocks (the first pair
// whose exclusive prefix reaches total * k / parts starts range k).
// Synchronises s.
size_t share_scratch_bytes(uint32_t count);
int share_range(const uint32_t *lens, const uint2 *pairs, uint32_t count, uint32_t identity,
                uint32_t part, uint32_t parts, void *scratch, uint32_t h_cut[2],
                cudaStream_t s);
size_t emit_scratch_bytes(uint32_t count, uint32_t n_nodes);
int emit_sorted(const uint2 *pairs, const uint32_t *scores, uint32_t count,
                uint32_t n_nodes, ngia_edge *out, uint64_t *h_m, void *scratch,
                cudaStream_t s);
int fast_round(const uint32_t *packed, const uint64_t *offs, const uint32_t *rep_row,
               uint32_t *parent, uint32_t n, uint32_t identity, uint32_t *jobs,
               uint32_t *d_count, cudaStream_t s);

}  // namespace ngia
