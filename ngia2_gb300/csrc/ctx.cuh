// ctx.cuh -- the resident-database context behind the opaque ngia_ctx of the
// C ABI (internal header; ctx.cu and serve.cu).
#pragma once

#include "round.cuh"

struct ngia_ctx {
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // 0-3 graph-build stage timing, 5 copy ordering, 6-7 fork/join of `side`,
  // 8-10 sketch and bucket timing
  static constexpr int kEvents = 11;
  cudaEvent_t ev[kEvents] = {};
  uint32_t *h_flag = nullptr;  // pinned: a pipelined load's check, read after the step
  cudaStream_t side = nullptr;  // work that runs beside the main stream's (sketch)
  // pipelined loads (ngia_ctx_run_host): chunks of the records copied on `copy`
  // while the previous chunks are sketched on `stream`
  static constexpr int kLoadChunks = 8;  // at most
  cudaStream_t copy = nullptr, layout = nullptr;  // copies; each piece's layouts
  cudaEvent_t chunk_ev[kLoadChunks] = {}, layout_ev[kLoadChunks] = {};
  uint32_t last_present = 0;  // residue codes of the previous load (0: none yet)
  // resident database
  uint32_t n = 0;
  uint64_t packed_words = 0;
  uint32_t rep_bands = 0;
  ngia::DevBuf packed, nib, offs, lens, rep, sigs;
  // the pieced load (ngia_ctx_run_host) writes no residue-code nibbles;
  // ctx_ready_layouts rebuilds them for the kernels that read them
  bool nib_stale = false;
  ngia::DevBuf staging;  // residue text of a load from text (released after it)
  ngia::DevBuf part_tmp;  // band blocks and their prefix (a graph build split over devices)
  bool sigs_valid = false;  // sigs hold all 64 bands of the loaded records
  // targets as the aligner reads them: densely recoded when the database uses
  // at most 7 nonzero residue codes (aligner tables of 8 entries), else `nib`
  ngia::DevBuf nib_dense, presence;
  ngia::DevBuf dplanes;  // recoded databases: planes of the aligner codes
  const uint32_t *align_nib = nullptr;
  ngia::Alphabet ab{16, 0xFEDCBA9876543210ull};
  uint64_t recode_map = 0;  // nibble c = aligner code of residue code c (when dense)
  // at most four residue codes, none of them 0: the sketch reads the 64 band
  // hashes of every 8-mer from a table (built on first use after a load)
  bool table_ok = false, table_built = false, use_table = true;
  uint64_t table_inv = 0;  // the aligner-code map the sketch tables were built for
  ngia::DevBuf sketch_table;
  // graph build work
  ngia::DevBuf ucount, uoff, counters, pairs, scores, emit_tmp, edges, scan_tmp, jobs,
      sort_tmp;
  uint64_t n_edges = 0;
  // the batched aligner (scratch, side streams, plan, cached graph) on `stream`
  ngia::Round round;
  // the bucketing's launches (partition passes, resolve) captured as one graph
  // and replayed while its buffers, n and bands stay the same: at small n its
  // dozen short launches cost more to issue than to run
  cudaGraphExec_t bucket_exec = nullptr;
  uint32_t bucket_kernels = 0;  // kernel nodes of bucket_exec
  const void *bucket_key[3] = {};
  uint64_t bucket_key_n = 0, bucket_key_gen = 0;
};

namespace ngia {
DbView db_view(const ngia_ctx *c);
// sketch_done: the signatures are already in place (a pipelined load).
// defer_stats: no wait for the stage timings; a later synchronisation makes
// them readable (ctx_stage_stats).
int ctx_sketch_bucket(ngia_ctx *c, uint32_t bands, ngia_stats *st, bool sketch_done = false,
                      bool defer_stats = false);
// ms_sketch and ms_bucket of the last ctx_sketch_bucket, once its work is done.
void ctx_stage_stats(ngia_ctx *c, ngia_stats *st);
// Rebuilds the residue-code nibbles a pieced load left out (on the
// context's stream), for the kernels that read them.
int ctx_ready_layouts(ngia_ctx *c);
int ctx_fast_cluster(ngia_ctx *c, uint32_t identity, uint32_t bands, uint32_t *h_cluster,
                     ngia_stats *st);
// Load from residue text (makedb): record i's h_lens[i] residues start at byte
// h_starts[i] of h_text; the device packs them into planes at word offsets
// h_offs[i] (`words` in all) and writes the nibble layout in the same pass.
int ctx_load_text(ngia_ctx *c, const char *h_text, uint64_t text_bytes,
                  const uint64_t *h_starts, const uint32_t *h_lens, const uint64_t *h_offs,
                  uint32_t n, uint64_t words);
// parts > 1: only the part-th share of the distinct pairs by band cells is
// aligned and emitted; h_range (optional) receives its [first, end).
int ctx_build_graph(ngia_ctx *c, uint32_t identity, uint32_t bands, uint64_t *h_n_edges,
                    ngia_stats *st, uint32_t part = 0, uint32_t parts = 1,
                    uint64_t *h_range = nullptr);
}  // namespace ngia
