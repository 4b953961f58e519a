// ctx.cu -- the resident-database context (ngia_ctx), the batched graph build
// and fast-mode driver, status handling, and the edge sort+unique entry point.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <vector>

#include "align.cuh"
#include "ctx.cuh"
#include "host.hpp"
#include "kernels.cuh"

namespace ngia {

static thread_local int g_last_cuda = 0;
static int g_round_mode = NGIA_ROUND_FMA;

int cuda_fail(cudaError_t e) {
  g_last_cuda = (int)e;
  (void)cudaGetLastError();  // clear a sticky-free error so later calls can run
  return e == cudaErrorMemoryAllocation ? NGIA_ERR_NOMEM : NGIA_ERR_CUDA;
}

int round_mode() { return g_round_mode; }

static std::atomic<unsigned long long> g_launches(0);
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_launches(long long delta) {
  g_launches.fetch_add((unsigned long long)delta, std::memory_order_relaxed);
}

}  // namespace ngia

namespace ngia {

DbView db_view(const ngia_ctx *c) {
  return DbView{c->packed.as<uint32_t>(), c->align_nib, c->ab, c->offs.as<uint64_t>(),
                c->lens.as<uint32_t>()};
}

// The bucketing on the context's stream, through a cached graph when the
// round uses graphs (captured again when the signature rows, rep rows or
// scratch move, or n or bands change).
static int bucket_graph(ngia_ctx *c, uint32_t bands) {
  cudaStream_t s = c->stream;
  if (!c->round.use_graphs)
    return bucket(c->sigs.as<uint32_t>(), c->n, bands, c->rep.as<uint32_t>(), c->sort_tmp.p, s);
  const uint64_t key_n = ((uint64_t)c->n << 8) | bands;
  const uint64_t gen = g_alloc_gen.load();
  if (!c->bucket_exec || c->bucket_key[0] != c->sigs.p || c->bucket_key[1] != c->rep.p ||
      c->bucket_key[2] != c->sort_tmp.p || c->bucket_key_n != key_n ||
      c->bucket_key_gen != gen) {
    if (c->bucket_exec) cudaGraphExecDestroy(c->bucket_exec);
    c->bucket_exec = nullptr;
    NGIA_TRY(sort_prepare());  // one-time attributes, outside the capture
    NGIA_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    int rc = bucket(c->sigs.as<uint32_t>(), c->n, bands, c->rep.as<uint32_t>(), c->sort_tmp.p, s);
    cudaGraph_t graph = nullptr;
    const cudaError_t e1 = cudaStreamEndCapture(s, &graph);
    if (rc == NGIA_OK && e1 != cudaSuccess) rc = cuda_fail(e1);
    if (rc == NGIA_OK) rc = instantiate_counted(graph, &c->bucket_exec, &c->bucket_kernels);
    if (graph) cudaGraphDestroy(graph);
    if (rc != NGIA_OK) {
      c->bucket_exec = nullptr;
      return rc;
    }
    c->bucket_key[0] = c->sigs.p;
    c->bucket_key[1] = c->rep.p;
    c->bucket_key[2] = c->sort_tmp.p;
    c->bucket_key_n = key_n;
    c->bucket_key_gen = gen;
  }
  NGIA_CUDA(cudaGraphLaunch(c->bucket_exec, s));
  note_launches(c->bucket_kernels);
  return NGIA_OK;
}

int ctx_ready_layouts(ngia_ctx *c) {
  if (c->nib_stale && c->n) {
    NGIA_TRY(c->presence.reserve(2 * sizeof(uint32_t)));  // word 1: scratch for the checks
    NGIA_TRY(launch_nibbles(c->packed.as<uint32_t>(), c->offs.as<uint64_t>(),
                            c->lens.as<uint32_t>(), c->n, c->packed_words,
                            c->nib.as<uint32_t>(), c->presence.as<uint32_t>() + 1, c->stream));
    c->nib_stale = false;
  }
  return NGIA_OK;
}

void ctx_stage_stats(ngia_ctx *c, ngia_stats *st) {
  st->ms_sketch = ev_ms(c->ev[8], c->ev[9]);
  st->ms_bucket = ev_ms(c->ev[9], c->ev[10]);
}

int ctx_sketch_bucket(ngia_ctx *c, uint32_t bands, ngia_stats *st, bool sketch_done,
                      bool defer_stats) {
  if (c->n == 0) return NGIA_ERR_STATE;
  if (bands < 1 || bands > (uint32_t)kBands) return NGIA_ERR_ARG;
  cudaStream_t s = c->stream;
  NGIA_TRY(c->sigs.reserve((size_t)kBands * c->n * 4));
  NGIA_TRY(c->rep.reserve((size_t)kBands * c->n * 4));
  NGIA_TRY(c->sort_tmp.reserve(bucket_scratch_bytes(c->n, bands)));
  // the tables depend only on the aligner-code map: built once per map
  if (!sketch_done && c->use_table && c->table_ok &&
      !(c->table_built && c->table_inv == c->ab.inv)) {
    NGIA_TRY(c->sketch_table.reserve(sketch_table_bytes()));
    NGIA_TRY(build_sketch_table(c->ab.inv, c->sketch_table.p, s));
    c->table_built = true;
    c->table_inv = c->ab.inv;
  }
  if (!sketch_done) {  // (else ev[8], ev[9] bracket the pipelined load and sketch)
    NGIA_CUDA(cudaEventRecord(c->ev[8], s));
    if (c->use_table && c->table_ok)
      NGIA_TRY(launch_sketch_table(c->packed.as<uint32_t>(), c->nib_dense.as<uint32_t>(),
                                   c->offs.as<uint64_t>(), c->n, c->packed_words, c->ab.inv,
                                   c->sketch_table.p,
                                   c->sigs.as<uint32_t>(), c->n, s, c->side, c->ev[6],
                                   c->ev[7]));
    else {
      NGIA_TRY(ctx_ready_layouts(c));  // a pieced load leaves the nibbles out
      NGIA_TRY(launch_sketch_nibbles(c->nib.as<uint32_t>(), c->offs.as<uint64_t>(), c->n,
                                     c->sigs.as<uint32_t>(), s));
    }
    NGIA_CUDA(cudaEventRecord(c->ev[9], s));
  }
  NGIA_TRY(bucket_graph(c, bands));
  NGIA_CUDA(cudaEventRecord(c->ev[10], s));
  c->rep_bands = bands;
  c->sigs_valid = true;
  if (st && !defer_stats) {
    NGIA_CUDA(cudaEventSynchronize(c->ev[10]));
    ctx_stage_stats(c, st);
  }
  return NGIA_OK;
}

int ctx_build_graph(ngia_ctx *c, uint32_t identity, uint32_t bands, uint64_t *h_n_edges,
                    ngia_stats *st, uint32_t part, uint32_t parts, uint64_t *h_range) {
  if (c->n == 0 || c->rep_bands == 0) return NGIA_ERR_STATE;
  if (identity < 1 || identity > 99) return NGIA_ERR_ARG;
  if (bands < 1 || bands > c->rep_bands) return NGIA_ERR_ARG;
  cudaStream_t s = c->stream;
  const uint32_t n = c->n;
  const uint32_t *rep = c->rep.as<uint32_t>();
  const uint32_t *lens = c->lens.as<uint32_t>();
  NGIA_TRY(c->counters.reserve(sizeof(Counters)));
  NGIA_TRY(c->ucount.reserve((size_t)n * 4));
  NGIA_TRY(c->uoff.reserve((size_t)n * 8));
  Counters *dc = c->counters.as<Counters>();
  NGIA_CUDA(cudaMemsetAsync(dc, 0, sizeof(Counters), s));
  NGIA_CUDA(cudaEventRecord(c->ev[0], s));
  // 1. candidates: distinct pairs grouped by target, in one pass (the pair
  // buffer holds the worst case, bands x n)
  NGIA_TRY(c->pairs.reserve((size_t)bands * n * 8));
  uint2 *pairs = c->pairs.as<uint2>();
  NGIA_TRY(collect_scan(rep, lens, n, bands, identity, &dc->collect_ticket,
                        reinterpret_cast<unsigned long long *>(c->uoff.p), &dc->cand_total,
                        &dc->unique_total, &dc->collect_error, pairs, s));
  Counters hc;
  NGIA_CUDA(cudaMemcpyAsync(&hc, dc, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  if (hc.collect_error) return NGIA_ERR_CUDA;  // a look-back gave up (never seen)
  const uint64_t total = hc.unique_total;
  if (total > 0xFFFFFFFFull) return NGIA_ERR_NOMEM;  // beyond one launch's index range
  uint32_t cut[2] = {0u, (uint32_t)total};
  if (parts > 1) {  // this device's share of the pairs, by band cells
    NGIA_TRY(c->part_tmp.reserve(share_scratch_bytes((uint32_t)total)));
    NGIA_TRY(share_range(lens, pairs, (uint32_t)total, identity, part, parts, c->part_tmp.p, cut,
                         s));
    pairs += cut[0];
  }
  if (h_range) {
    h_range[0] = cut[0];
    h_range[1] = cut[1];
  }
  const uint32_t m = cut[1] - cut[0];
  NGIA_TRY(c->scores.reserve((size_t)(m ? m : 1) * 4));
  uint32_t *scores = c->scores.as<uint32_t>();
  // 2-3. width classes, then one persistent launch per class (the round is
  // on the context's stream)
  NGIA_TRY(c->round.reserve(m));
  NGIA_TRY(c->round.enqueue(db_view(c), pairs, m, identity, scores, c->ev[1]));
  NGIA_CUDA(cudaEventRecord(c->ev[2], s));
  // 4. emit: compact hits, sort by (rep, tar)
  NGIA_TRY(c->emit_tmp.reserve(emit_scratch_bytes(m, n)));
  NGIA_TRY(c->edges.reserve((size_t)(m ? m : 1) * sizeof(ngia_edge)));
  uint64_t ne = 0;
  NGIA_TRY(emit_sorted(pairs, scores, m, n, c->edges.as<ngia_edge>(), &ne, c->emit_tmp.p, s));
  NGIA_CUDA(cudaEventRecord(c->ev[3], s));
  NGIA_CUDA(cudaEventSynchronize(c->ev[3]));
  c->n_edges = ne;
  if (h_n_edges) *h_n_edges = ne;
  if (st) {
    Counters rc;
    NGIA_CUDA(cudaMemcpy(&rc, c->round.counters(), sizeof(Counters), cudaMemcpyDeviceToHost));
    st->candidate_pairs = hc.cand_total;
    st->unique_pairs = m;
    st->aligned_cells = rc.cells;
    st->computed_cells = rc.work * 1024ull;
    st->edges = ne;
    st->ms_pairs = ev_ms(c->ev[0], c->ev[1]);
    st->ms_align = ev_ms(c->ev[1], c->ev[2]);
    st->ms_emit = ev_ms(c->ev[2], c->ev[3]);
  }
  return NGIA_OK;
}

// The batched aligner on caller-given pairs (device arrays) of the resident
// database.  Every index must be below the record count.  With graphs on, the
// round is captured once per (pairs, scores, count, identity, rounding,
// allocations, plan) and replayed.
int ctx_align_pairs(ngia_ctx *c, const uint2 *d_pairs, uint32_t m, uint32_t identity,
                    uint32_t *d_scores, ngia_stats *st) {
  if (c->n == 0) return NGIA_ERR_STATE;
  if (identity < 1 || identity > 99) return NGIA_ERR_ARG;
  if (st) std::memset(st, 0, sizeof(*st));
  RoundStats rs;
  NGIA_TRY(c->round.run(db_view(c), d_pairs, m, identity, d_scores, &rs));
  if (st) {
    st->candidate_pairs = m;
    st->unique_pairs = m;
    st->aligned_cells = rs.cells;
    st->computed_cells = rs.work * 1024ull;
    st->ms_pairs = rs.ms_classify;
    st->ms_align = rs.ms_align;
  }
  return NGIA_OK;
}

int ctx_fast_cluster(ngia_ctx *c, uint32_t identity, uint32_t bands, uint32_t *h_cluster,
                     ngia_stats *st) {
  if (c->n == 0 || c->rep_bands == 0) return NGIA_ERR_STATE;
  if (identity < 1 || identity > 99) return NGIA_ERR_ARG;
  if (bands < 1 || bands > c->rep_bands) return NGIA_ERR_ARG;
  cudaStream_t s = c->stream;
  const uint32_t n = c->n;
  NGIA_TRY(c->counters.reserve(sizeof(Counters)));
  NGIA_TRY(c->jobs.reserve((size_t)n * 12));
  NGIA_TRY(c->ucount.reserve((size_t)n * 4));  // parent pointers
  uint32_t *parent = c->ucount.as<uint32_t>();
  Counters *dc = c->counters.as<Counters>();
  NGIA_CUDA(cudaMemsetAsync(parent, 0xFF, (size_t)n * 4, s));
  NGIA_CUDA(cudaEventRecord(c->ev[0], s));
  for (uint32_t b = 0; b < bands; ++b)
    NGIA_TRY(fast_round(c->packed.as<uint32_t>(), c->offs.as<uint64_t>(),
                        c->rep.as<uint32_t>() + (size_t)b * n, parent, n, identity,
                        c->jobs.as<uint32_t>(), &dc->fast_count, s));
  NGIA_CUDA(cudaEventRecord(c->ev[1], s));
  std::vector<uint32_t> par(n);
  NGIA_CUDA(cudaMemcpyAsync(par.data(), parent, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  // Root resolution (src/fastClustering.hpp:338-347): parents precede children.
  for (uint32_t i = 0; i < n; ++i)
    h_cluster[i] = par[i] == kFull ? i : h_cluster[par[i]];
  if (st) {
    std::memset(st, 0, sizeof(*st));
    st->ms_align = ev_ms(c->ev[0], c->ev[1]);
  }
  return NGIA_OK;
}

// Dense recoding of the residue codes in use (code 0 stays 0): equality of
// codes, all the aligner looks at, is unchanged by a bijection.
struct AlphaChoice {
  bool dense = false;
  uint64_t map = 0, inv = 0;
  int K = 16;
  bool table_ok = false;
  bool operator==(const AlphaChoice &o) const {
    return dense == o.dense && map == o.map && inv == o.inv && K == o.K && table_ok == o.table_ok;
  }
};

static AlphaChoice choose_alphabet(uint32_t present) {
  AlphaChoice a;
  a.table_ok = (present & 1u) == 0 && present != 0 && __builtin_popcount(present) <= 4;
  if (__builtin_popcount(present & ~1u) <= 7) {
    int next = 1;
    for (int code = 1; code < 16; ++code) {
      if (!((present >> code) & 1u)) continue;
      a.map |= (uint64_t)next << (4 * code);
      a.inv |= (uint64_t)code << (4 * next);
      ++next;
    }
    a.dense = true;
    a.K = next <= 5 ? 5 : 8;
  }
  return a;
}

// Makes `a` the context's alphabet; with `layouts`, writes the recoded
// nibbles and code planes of all n records (dense alphabets).
static int use_alphabet(ngia_ctx *c, const AlphaChoice &a, uint64_t words, uint32_t n,
                        bool layouts) {
  c->table_ok = a.table_ok;
  c->align_nib = c->nib.as<uint32_t>();
  c->ab = Alphabet{16, 0xFEDCBA9876543210ull};
  c->recode_map = 0;
  if (!a.dense) return NGIA_OK;
  NGIA_TRY(c->nib_dense.reserve(words * 4));
  NGIA_TRY(c->dplanes.reserve(words * 4));
  if (layouts)
    NGIA_TRY(launch_dense_layouts(c->packed.as<uint32_t>(), c->offs.as<uint64_t>(), n, a.map,
                                  c->nib_dense.as<uint32_t>(), c->dplanes.as<uint32_t>(),
                                  c->stream));
  c->align_nib = c->nib_dense.as<uint32_t>();
  c->ab = Alphabet{a.K, a.inv, c->dplanes.as<uint32_t>()};
  c->recode_map = a.map;
  return NGIA_OK;
}

// Every record inside the region by its offset and read length, and no read
// longer than the format allows (one pass over the two arrays, before any
// copy); the device checks each record's length word as it lays it out.
bool records_inside(const uint64_t *h_offs, const uint32_t *h_lens, uint32_t n,
                    uint64_t words) {
  // the longest read and the furthest record end, compared once (a max
  // reduction the compiler vectorises; a record's end lies past its offset)
  uint32_t max_len = 0;
  uint64_t max_end = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t len = h_lens[i];
    const uint64_t end = h_offs[i] + 1 + 4ull * (((uint64_t)len + 31u) >> 5);
    max_len = len > max_len ? len : max_len;
    max_end = end > max_end ? end : max_end;
  }
  return max_len <= NGIA_MAX_READ && max_end <= words;
}

int ctx_load(ngia_ctx *c, const uint32_t *h_packed, uint64_t words, const uint64_t *h_offs,
             const uint32_t *h_lens, uint32_t n, const uint32_t *h_rep, uint32_t bands) {
  if (n == 0 || !h_packed || !h_offs || !h_lens) return NGIA_ERR_ARG;
  if (h_rep && (bands < 1 || bands > (uint32_t)kBands)) return NGIA_ERR_ARG;
  if (!records_inside(h_offs, h_lens, n, words)) return NGIA_ERR_ARG;
  cudaStream_t s = c->stream;
  NGIA_TRY(c->packed.reserve(words * 4));
  NGIA_TRY(c->offs.reserve((size_t)n * 8));
  NGIA_TRY(c->lens.reserve((size_t)n * 4));
  NGIA_CUDA(cudaMemcpyAsync(c->packed.p, h_packed, words * 4, cudaMemcpyHostToDevice, s));
  NGIA_CUDA(cudaMemcpyAsync(c->offs.p, h_offs, (size_t)n * 8, cudaMemcpyHostToDevice, s));
  NGIA_CUDA(cudaMemcpyAsync(c->lens.p, h_lens, (size_t)n * 4, cudaMemcpyHostToDevice, s));
  NGIA_TRY(c->nib.reserve(words * 4));
  NGIA_TRY(c->presence.reserve(sizeof(uint32_t)));
  NGIA_TRY(launch_nibbles(c->packed.as<uint32_t>(), c->offs.as<uint64_t>(),
                          c->lens.as<uint32_t>(), n, words, c->nib.as<uint32_t>(),
                          c->presence.as<uint32_t>(), s));
  c->nib_stale = false;
  uint32_t present = 0;
  NGIA_CUDA(cudaMemcpyAsync(&present, c->presence.p, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  if (present & kBadRecord) {  // a length word that is not the record's read length
    c->n = 0;
    return NGIA_ERR_FORMAT;
  }
  NGIA_TRY(use_alphabet(c, choose_alphabet(present), words, n, true));
  c->last_present = present;
  c->n = n;
  c->sigs_valid = false;
  c->packed_words = words;
  c->rep_bands = 0;
  c->n_edges = 0;
  if (h_rep) {
    NGIA_TRY(c->rep.reserve((size_t)kBands * n * 4));
    NGIA_CUDA(cudaMemcpyAsync(c->rep.p, h_rep, (size_t)bands * n * 4,
                              cudaMemcpyHostToDevice, s));
    c->rep_bands = bands;
  }
  return NGIA_OK;
}

int ctx_load_text(ngia_ctx *c, const char *h_text, uint64_t text_bytes,
                  const uint64_t *h_starts, const uint32_t *h_lens, const uint64_t *h_offs,
                  uint32_t n, uint64_t words) {
  if (n == 0 || !h_text || !h_starts || !h_lens || !h_offs) return NGIA_ERR_ARG;
  cudaStream_t s = c->stream;
  NGIA_TRY(c->packed.reserve(words * 4));
  NGIA_TRY(c->nib.reserve(words * 4));
  NGIA_TRY(c->offs.reserve((size_t)n * 8));
  NGIA_TRY(c->lens.reserve((size_t)n * 4));
  NGIA_TRY(c->presence.reserve(sizeof(uint32_t)));
  const size_t starts_at = (text_bytes + 15) & ~(size_t)15;
  NGIA_TRY(c->staging.reserve(starts_at + (size_t)n * 8));
  char *d_text = c->staging.as<char>();
  uint64_t *d_starts = reinterpret_cast<uint64_t *>(d_text + starts_at);
  NGIA_CUDA(cudaMemcpyAsync(d_text, h_text, text_bytes, cudaMemcpyHostToDevice, s));
  NGIA_CUDA(cudaMemcpyAsync(d_starts, h_starts, (size_t)n * 8, cudaMemcpyHostToDevice, s));
  NGIA_CUDA(cudaMemcpyAsync(c->offs.p, h_offs, (size_t)n * 8, cudaMemcpyHostToDevice, s));
  NGIA_CUDA(cudaMemcpyAsync(c->lens.p, h_lens, (size_t)n * 4, cudaMemcpyHostToDevice, s));
  NGIA_TRY(launch_pack_layout(reinterpret_cast<const uint8_t *>(d_text), d_starts,
                              c->lens.as<uint32_t>(), n, c->offs.as<uint64_t>(),
                              c->packed.as<uint32_t>(), c->nib.as<uint32_t>(),
                              c->presence.as<uint32_t>(), s));
  c->nib_stale = false;
  uint32_t present = 0;
  NGIA_CUDA(cudaMemcpyAsync(&present, c->presence.p, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  c->staging.release();
  NGIA_TRY(use_alphabet(c, choose_alphabet(present), words, n, true));
  c->last_present = present;
  c->n = n;
  c->sigs_valid = false;
  c->packed_words = words;
  c->rep_bands = 0;
  c->n_edges = 0;
  return NGIA_OK;
}

int makedb_device(ngia_ctx *c, Makedb &m) {
  if (!c || m.n == 0 || !m.file.data) return NGIA_ERR_ARG;
  cudaStream_t s = c->stream;
  NGIA_TRY(ctx_load_text(c, m.file.data + m.fasta0, m.size - m.fasta0, m.text_starts.data(),
                         m.lens.data(), m.offsets.data(), m.n, m.words));
  NGIA_TRY(ctx_sketch_bucket(c, kBands, nullptr));
  // the 64 rep rows (band-major) over the signature area, then the planes
  NGIA_CUDA(cudaMemcpyAsync(m.file.data + sig_area_offset(m.n), c->rep.p,
                            (size_t)kBands * m.n * 4, cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaMemcpyAsync(m.file.data + m.pack0, c->packed.p, m.words * 4,
                            cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  return NGIA_OK;
}

// Load and sketch in one pipeline (ngia_ctx_run_host): the records go to the
// device in pieces on their own stream, and each piece's layouts and
// signatures are computed while the next pieces are in flight.  The layouts
// and the sketch need the database's code map, known only once every record
// has been seen; the pipeline assumes the previous load's map (its sketch
// tables are cached) and checks that every residue's code is one of the map's
// and every record lay inside its piece (offsets in order); the check's
// result lands in *c->h_flag (nonzero: the caller discards the step and loads
// as usual) once the stream passes it.  Runs only when that map takes the
// table sketch.  *used = false: nothing was done (the caller loads as usual);
// else the load and the signatures are in place, subject to the check.
int ctx_load_sketch(ngia_ctx *c, const uint32_t *h_packed, uint64_t words,
                    const uint64_t *h_offs, const uint32_t *h_lens, uint32_t n, bool *used,
                    bool *sketched) {
  *used = *sketched = false;
  if (!c->h_flag) {  // pinned, so that the check's copy stays asynchronous
    void *p = nullptr;
    if (cudaHostAlloc(&p, sizeof(uint32_t), cudaHostAllocDefault) != cudaSuccess) {
      (void)cudaGetLastError();
      return NGIA_OK;  // the plain load then
    }
    c->h_flag = static_cast<uint32_t *>(p);
  }
  if (n < 4096 || !h_packed || !h_offs || !h_lens || !c->last_present || !c->use_table)
    return NGIA_OK;
  const AlphaChoice spec = choose_alphabet(c->last_present);
  if (!spec.dense || !spec.table_ok || !c->table_built || c->table_inv != spec.inv)
    return NGIA_OK;
  *used = true;
  cudaStream_t s = c->stream;
  NGIA_TRY(c->packed.reserve(words * 4));
  NGIA_TRY(c->offs.reserve((size_t)n * 8));
  NGIA_TRY(c->lens.reserve((size_t)n * 4));
  NGIA_TRY(c->nib.reserve(words * 4));
  NGIA_TRY(c->nib_dense.reserve(words * 4));
  NGIA_TRY(c->dplanes.reserve(words * 4));
  NGIA_TRY(c->presence.reserve(2 * sizeof(uint32_t)));
  NGIA_TRY(c->sigs.reserve((size_t)kBands * n * 4));
  NGIA_CUDA(cudaMemcpyAsync(c->offs.p, h_offs, (size_t)n * 8, cudaMemcpyHostToDevice, s));
  NGIA_CUDA(cudaMemcpyAsync(c->lens.p, h_lens, (size_t)n * 4, cudaMemcpyHostToDevice, s));
  NGIA_CUDA(cudaMemsetAsync(c->presence.p, 0, sizeof(uint32_t), s));
  // pieces cut at record boundaries, taken from the end of the buffer and
  // growing (the last 1/8 of the words, the 1/8 before, then 1/4, then the
  // first half): the first copy, which nothing hides, is short, the later
  // sketch launches have enough records per warp, and the shortest records
  // (length order), whose signatures come from the short records' kernel on
  // the side stream, arrive first, so that kernel runs beside the rest of the
  // pipeline.  The cuts assume offsets in order; the layout kernel verifies
  // every record lies in its piece.
  constexpr uint32_t kCuts[] = {4, 8, 12, 14};  // cut points, in sixteenths of the words
  constexpr int C = (int)(sizeof(kCuts) / sizeof(kCuts[0])) + 1;
  static_assert(C <= ngia_ctx::kLoadChunks, "pieces");
  uint32_t first[C + 1];
  uint64_t cut[C + 1];
  cut[0] = 0;
  for (int k = 1; k < C; ++k) cut[k] = words / 16 * kCuts[k - 1];
  cut[C] = words;
  first[0] = 0;
  for (int k = 1; k < C; ++k) {
    const uint64_t *p = std::lower_bound(h_offs, h_offs + n, cut[k]);
    first[k] = (uint32_t)(p - h_offs);
    if (first[k] < first[k - 1]) first[k] = first[k - 1];
  }
  first[C] = n;
  uint32_t *packed = c->packed.as<uint32_t>();
  // piece k's words: [bound(k), bound(k + 1)), inside the region whatever the
  // offsets hold.  Nothing launched here trusts the offsets: the layout
  // kernel checks every record against its piece and the sketch bounds every
  // record by the region; the caller checks them on the host while this runs
  // (ngia_ctx_run_host) and before anything that trusts them is launched.
  auto bound = [&](int k) -> uint64_t {
    if (k <= 0) return 0;
    if (k >= C) return words;
    const uint64_t w = first[k] < n ? h_offs[first[k]] : words;
    return w < words ? w : words;
  };
  // the copies overwrite records that earlier work on the stream may still read
  NGIA_CUDA(cudaEventRecord(c->ev[5], s));
  NGIA_CUDA(cudaStreamWaitEvent(c->copy, c->ev[5], 0));
  for (int k = C - 1; k >= 0; --k) {
    const uint64_t w0 = bound(k), w1 = bound(k + 1);
    if (w1 > w0)
      NGIA_CUDA(cudaMemcpyAsync(packed + w0, h_packed + w0, (w1 - w0) * 4,
                                cudaMemcpyHostToDevice, c->copy));
    NGIA_CUDA(cudaEventRecord(c->chunk_ev[k], c->copy));
  }
  // each piece's layouts on their own stream right behind its copy, so they
  // can run while the main stream sketches the previous piece
  const uint64_t *offs = c->offs.as<uint64_t>();
  for (int k = C - 1; k >= 0; --k) {
    const uint32_t r0 = first[k], cnt = first[k + 1] - first[k];
    NGIA_CUDA(cudaStreamWaitEvent(c->layout, c->chunk_ev[k], 0));
    if (cnt) {
      const uint64_t w0 = bound(k), w1 = bound(k + 1);
      NGIA_TRY(launch_load_layouts(packed, offs + r0, c->lens.as<uint32_t>() + r0, cnt, w0, w1,
                                   words, spec.inv, c->nib_dense.as<uint32_t>(),
                                   c->dplanes.as<uint32_t>(), c->presence.as<uint32_t>(),
                                   c->layout));
    }
    NGIA_CUDA(cudaEventRecord(c->layout_ev[k], c->layout));
  }
  NGIA_CUDA(cudaEventRecord(c->ev[8], s));
  for (int k = C - 1; k >= 0; --k) {
    const uint32_t r0 = first[k], cnt = first[k + 1] - first[k];
    NGIA_CUDA(cudaStreamWaitEvent(s, c->layout_ev[k], 0));
    if (cnt == 0) continue;
    NGIA_TRY(launch_sketch_table(packed, c->nib_dense.as<uint32_t>(), offs + r0,
                                 cnt, words, spec.inv, c->sketch_table.p,
                                 c->sigs.as<uint32_t>() + r0, n, s, c->side, c->ev[6], nullptr));
  }
  NGIA_CUDA(cudaEventRecord(c->ev[7], c->side));  // the short records' kernels
  NGIA_CUDA(cudaStreamWaitEvent(s, c->ev[7], 0));
  NGIA_CUDA(cudaEventRecord(c->ev[9], s));
  // a code outside the map, or a record outside its piece: copied to
  // *h_flag and read by the caller after the step's next synchronisation,
  // without a host round trip here.  Until then the step goes on as if the map serves (the
  // layouts of such records hold in-range codes, so the work on them is
  // wasted, never out of bounds); if the check fails, the caller starts over
  // with the plain load.
  *c->h_flag = 0;
  NGIA_CUDA(cudaMemcpyAsync(c->h_flag, c->presence.p, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            s));
  *sketched = true;
  c->nib_stale = true;
  NGIA_TRY(use_alphabet(c, spec, words, n, false));
  c->n = n;
  c->sigs_valid = false;
  c->packed_words = words;
  c->rep_bands = 0;
  c->n_edges = 0;
  return NGIA_OK;
}

}  // namespace ngia

// ---- C ABI --------------------------------------------------------------------------
extern "C" {

const char *ngia_status_string(int status) {
  switch (status) {
    case NGIA_OK: return "ok";
    case NGIA_ERR_ARG: return "invalid argument";
    case NGIA_ERR_CUDA: return "CUDA error";
    case NGIA_ERR_NOMEM: return "out of memory";
    case NGIA_ERR_IO: return "I/O error";
    case NGIA_ERR_FORMAT: return "malformed input";
    case NGIA_ERR_STATE: return "call out of order";
    default: return "unknown status";
  }
}

int ngia_last_cuda_error(void) { return ngia::g_last_cuda; }

unsigned long long ngia_kernel_launches(void) { return ngia::g_launches.load(); }

const char *ngia_version(void) { return "ngia-gb300 0.1 (sm_103a)"; }

int ngia_set_round_mode(int mode) {
  const int old = ngia::g_round_mode;
  if (mode == NGIA_ROUND_SPLIT || mode == NGIA_ROUND_FMA) ngia::g_round_mode = mode;
  return old;
}

int ngia_ctx_create(ngia_ctx **out, void *stream) {
  if (!out) return NGIA_ERR_ARG;
  *out = nullptr;
  ngia_ctx *c = new (std::nothrow) ngia_ctx();
  if (!c) return NGIA_ERR_NOMEM;
  cudaError_t e = cudaSuccess;
  if (stream) {
    c->stream = static_cast<cudaStream_t>(stream);
  } else {
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    c->own_stream = (e == cudaSuccess);
  }
  for (int k = 0; k < ngia_ctx::kEvents && e == cudaSuccess; ++k) e = cudaEventCreate(&c->ev[k]);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->layout, cudaStreamNonBlocking);
  for (int k = 0; k < ngia_ctx::kLoadChunks && e == cudaSuccess; ++k) {
    e = cudaEventCreateWithFlags(&c->chunk_ev[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->layout_ev[k], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    ngia_ctx_destroy(c);
    return ngia::cuda_fail(e);
  }
  const int rc = c->round.init(c->stream);
  if (rc != NGIA_OK) {
    ngia_ctx_destroy(c);
    return rc;
  }
  *out = c;
  return NGIA_OK;
}

void ngia_ctx_destroy(ngia_ctx *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  ngia::DevBuf *bufs[] = {&c->packed,   &c->nib,   &c->nib_dense, &c->dplanes,  &c->presence,
                          &c->staging,  &c->part_tmp,
                          &c->offs,     &c->lens,  &c->rep,       &c->sigs,     &c->ucount,
                          &c->uoff,
                          &c->counters, &c->pairs, &c->scores,    &c->sort_tmp, &c->emit_tmp,
                          &c->edges,    &c->scan_tmp, &c->jobs, &c->sketch_table};
  for (ngia::DevBuf *b : bufs) b->release();
  c->round.destroy();  // shares c->stream, which it leaves alone
  for (int k = 0; k < ngia_ctx::kEvents; ++k)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  if (c->h_flag) cudaFreeHost(c->h_flag);
  c->h_flag = nullptr;
  if (c->bucket_exec) cudaGraphExecDestroy(c->bucket_exec);
  c->bucket_exec = nullptr;
  if (c->side) cudaStreamDestroy(c->side);
  if (c->copy) cudaStreamDestroy(c->copy);
  if (c->layout) cudaStreamDestroy(c->layout);
  for (cudaEvent_t e : c->chunk_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : c->layout_ev)
    if (e) cudaEventDestroy(e);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int ngia_ctx_load(ngia_ctx *c, const uint32_t *h_packed, uint64_t packed_words,
                  const uint64_t *h_rec_offsets, const uint32_t *h_lens, uint32_t n,
                  const uint32_t *h_rep, uint32_t bands) {
  if (!c) return NGIA_ERR_ARG;
  NGIA_TRY(ngia::ctx_load(c, h_packed, packed_words, h_rec_offsets, h_lens, n, h_rep, bands));
  NGIA_CUDA(cudaStreamSynchronize(c->stream));
  return NGIA_OK;
}

int ngia_ctx_load_packed_file(ngia_ctx *c, const char *path, uint32_t bands,
                              int use_file_rep_rows) {
  if (!c || !path) return NGIA_ERR_ARG;
  if (bands < 1 || bands > NGIA_BANDS) return NGIA_ERR_ARG;
  ngia::PackedDb db;
  NGIA_TRY(ngia::read_packed(path, use_file_rep_rows ? bands : 0, db));
  NGIA_TRY(ngia::ctx_load(c, db.packed.data(), db.packed.size(), db.offsets.data(),
                          db.lens.data(), db.n, use_file_rep_rows ? db.rep.data() : nullptr,
                          bands));
  NGIA_CUDA(cudaStreamSynchronize(c->stream));
  if (!use_file_rep_rows) NGIA_TRY(ngia::ctx_sketch_bucket(c, bands, nullptr));
  return NGIA_OK;
}

int ngia_ctx_sketch_bucket(ngia_ctx *c, uint32_t bands) {
  if (!c) return NGIA_ERR_ARG;
  NGIA_TRY(ngia::ctx_sketch_bucket(c, bands, nullptr));
  NGIA_CUDA(cudaStreamSynchronize(c->stream));
  return NGIA_OK;
}

int ngia_ctx_build_graph(ngia_ctx *c, uint32_t identity, uint32_t bands,
                         uint64_t *h_n_edges, ngia_stats *stats) {
  if (!c) return NGIA_ERR_ARG;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  return ngia::ctx_build_graph(c, identity, bands, h_n_edges, stats);
}

int ngia_ctx_build_graph_part(ngia_ctx *c, uint32_t identity, uint32_t bands, uint32_t part,
                              uint32_t parts, uint64_t *h_range, uint64_t *h_n_edges,
                              ngia_stats *stats) {
  if (!c || parts < 1 || part >= parts) return NGIA_ERR_ARG;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  return ngia::ctx_build_graph(c, identity, bands, h_n_edges, stats, part, parts, h_range);
}

int ngia_ctx_group_align(ngia_ctx *c, uint32_t identity, uint32_t bands,
                         uint64_t *h_n_edges, ngia_stats *stats) {
  if (!c) return NGIA_ERR_ARG;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  // the stage timings are read after the graph build's synchronisation, so
  // that no host round trip sits between the bucketing and the candidates
  NGIA_TRY(ngia::ctx_sketch_bucket(c, bands, stats, false, true));
  NGIA_TRY(ngia::ctx_build_graph(c, identity, bands, h_n_edges, stats));
  if (stats) ngia::ctx_stage_stats(c, stats);
  return NGIA_OK;
}

int ngia_ctx_test_lookback_timeout(ngia_ctx *c, uint32_t identity, uint32_t bands,
                                   uint32_t spin_limit) {
  using namespace ngia;
  if (!c) return NGIA_ERR_ARG;
  if (c->n == 0 || c->rep_bands == 0) return NGIA_ERR_STATE;
  if (identity < 1 || identity > 99 || bands < 1 || bands > c->rep_bands) return NGIA_ERR_ARG;
  if (spin_limit < 1 || spin_limit > kLookbackSpins) return NGIA_ERR_ARG;
  cudaStream_t s = c->stream;
  const uint32_t n = c->n;
  NGIA_TRY(c->counters.reserve(sizeof(Counters)));
  NGIA_TRY(c->uoff.reserve((size_t)n * 8));
  NGIA_TRY(c->pairs.reserve((size_t)bands * n * 8));
  Counters *dc = c->counters.as<Counters>();
  NGIA_CUDA(cudaMemsetAsync(dc, 0, sizeof(Counters), s));
  const unsigned int one = 1;  // the first ticket handed out is 1: block 0 never publishes
  NGIA_CUDA(cudaMemcpyAsync(&dc->collect_ticket, &one, sizeof(one), cudaMemcpyHostToDevice, s));
  NGIA_TRY(collect_scan(c->rep.as<uint32_t>(), c->lens.as<uint32_t>(), n, bands, identity,
                        &dc->collect_ticket, reinterpret_cast<unsigned long long *>(c->uoff.p),
                        &dc->cand_total, &dc->unique_total, &dc->collect_error,
                        c->pairs.as<uint2>(), s, spin_limit));
  Counters hc;
  NGIA_CUDA(cudaMemcpyAsync(&hc, dc, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  return hc.collect_error ? NGIA_ERR_CUDA : NGIA_OK;
}

int ngia_ctx_edges(ngia_ctx *c, ngia_edge *h_edges, uint64_t cap) {
  if (!c || (!h_edges && cap)) return NGIA_ERR_ARG;
  const uint64_t m = c->n_edges < cap ? c->n_edges : cap;
  if (m == 0) return NGIA_OK;
  NGIA_CUDA(cudaMemcpyAsync(h_edges, c->edges.p, m * sizeof(ngia_edge),
                            cudaMemcpyDeviceToHost, c->stream));
  NGIA_CUDA(cudaStreamSynchronize(c->stream));
  return NGIA_OK;
}

int ngia_ctx_align_pairs(ngia_ctx *c, const uint32_t *d_pairs, uint32_t count,
                         uint32_t identity, uint32_t *d_scores, ngia_stats *stats) {
  if (!c || (count && (!d_pairs || !d_scores))) return NGIA_ERR_ARG;
  return ngia::ctx_align_pairs(c, reinterpret_cast<const uint2 *>(d_pairs), count, identity,
                               d_scores, stats);
}

static_assert(NGIA_GROUP_CLASSES == ngia::kNumGroupClasses, "plan layout");

static bool plan_valid(const ngia_plan &p) {
  if (p.stream_max < 4 || p.stream_max > 16) return false;
  for (int g = 0; g < NGIA_GROUP_CLASSES; ++g)
    if (p.group_limit[g] > ngia::group_span_limit(ngia::kFirstGroupClass + g)) return false;
  return true;
}

int ngia_ctx_get_plan(ngia_ctx *c, ngia_plan *p) {
  if (!c || !p) return NGIA_ERR_ARG;
  p->stream_max = c->round.plan.stream_max;
  for (int g = 0; g < NGIA_GROUP_CLASSES; ++g) p->group_limit[g] = c->round.plan.group_limit[g];
  return NGIA_OK;
}

int ngia_ctx_set_plan(ngia_ctx *c, const ngia_plan *p) {
  if (!c || !p || !plan_valid(*p)) return NGIA_ERR_ARG;
  c->round.plan.stream_max = p->stream_max;
  for (int g = 0; g < NGIA_GROUP_CLASSES; ++g) c->round.plan.group_limit[g] = p->group_limit[g];
  ++c->round.plan_gen;
  return NGIA_OK;
}

int ngia_ctx_autotune(ngia_ctx *c, const uint32_t *d_pairs, uint32_t count, uint32_t identity,
                      int reps, ngia_plan *best, double *best_ms) {
  if (!c || (count && !d_pairs)) return NGIA_ERR_ARG;
  if (c->n == 0) return NGIA_ERR_STATE;
  if (identity < 1 || identity > 99 || count == 0) return NGIA_ERR_ARG;
  if (reps < 1) reps = 1;
  NGIA_TRY(c->scores.reserve((size_t)count * 4));
  // timed the way the round runs (replayed as a graph when graphs are on; a
  // plan change recaptures, so the first of the reps carries the capture and
  // the best of them is kept)
  const uint2 *pairs = reinterpret_cast<const uint2 *>(d_pairs);
  auto time_plan = [&](const ngia_plan &p, double *ms) -> int {
    NGIA_TRY(ngia_ctx_set_plan(c, &p));
    double t_min = 1e30;
    for (int r = 0; r < reps; ++r) {
      ngia_stats st;
      NGIA_TRY(ngia::ctx_align_pairs(c, pairs, count, identity, c->scores.as<uint32_t>(), &st));
      const double t = st.ms_pairs + st.ms_align;
      if (t < t_min) t_min = t;
    }
    *ms = t_min;
    return NGIA_OK;
  };
  ngia_plan cur;
  ngia_ctx_get_plan(c, &cur);
  double t_cur = 0;
  int rc = time_plan(cur, &t_cur);
  // coordinate descent: the widest per-lane window, then each group class
  // on (at its largest band) or off; a move must win by 2 %
  for (int pass = 0; pass < 2 && rc == NGIA_OK; ++pass) {
    for (uint32_t sm = 8; sm <= 16 && rc == NGIA_OK; sm += 2) {
      if (sm == cur.stream_max) continue;
      ngia_plan p = cur;
      p.stream_max = sm;
      double t = 0;
      rc = time_plan(p, &t);
      if (rc == NGIA_OK && t < 0.98 * t_cur) {
        cur = p;
        t_cur = t;
      }
    }
    for (int g = 0; g < NGIA_GROUP_CLASSES && rc == NGIA_OK; ++g) {
      ngia_plan p = cur;
      const uint32_t lim = ngia::group_span_limit(ngia::kFirstGroupClass + g);
      p.group_limit[g] = cur.group_limit[g] ? 0u : lim;
      double t = 0;
      rc = time_plan(p, &t);
      if (rc == NGIA_OK && t < 0.98 * t_cur) {
        cur = p;
        t_cur = t;
      }
    }
  }
  if (rc != NGIA_OK) return rc;
  NGIA_TRY(ngia_ctx_set_plan(c, &cur));
  if (best) *best = cur;
  if (best_ms) *best_ms = t_cur;
  return NGIA_OK;
}

int ngia_ctx_use_sketch_table(ngia_ctx *c, int on) {
  if (!c) return NGIA_ERR_ARG;
  const int old = c->use_table ? 1 : 0;
  c->use_table = on != 0;
  return old;
}

int ngia_ctx_sketch_table_active(ngia_ctx *c) {
  if (!c) return NGIA_ERR_ARG;
  return c->use_table && c->table_ok ? 1 : 0;
}

int ngia_ctx_sigs(ngia_ctx *c, uint32_t *h_sigs) {
  if (!c || !h_sigs) return NGIA_ERR_ARG;
  if (!c->sigs_valid) return NGIA_ERR_STATE;
  NGIA_CUDA(cudaMemcpyAsync(h_sigs, c->sigs.p, (size_t)ngia::kBands * c->n * 4,
                            cudaMemcpyDeviceToHost, c->stream));
  NGIA_CUDA(cudaStreamSynchronize(c->stream));
  return NGIA_OK;
}

int ngia_ctx_use_graphs(ngia_ctx *c, int on) {
  if (!c) return NGIA_ERR_ARG;
  const int old = c->round.use_graphs ? 1 : 0;
  c->round.use_graphs = on != 0;
  return old;
}

int ngia_ctx_align_pairs_host(ngia_ctx *c, const uint32_t *h_pairs, uint32_t count,
                              uint32_t identity, uint32_t *h_scores, ngia_stats *stats) {
  if (!c || (count && (!h_pairs || !h_scores))) return NGIA_ERR_ARG;
  if (c->n == 0) return NGIA_ERR_STATE;
  for (uint64_t j = 0; j < 2ull * count; ++j)
    if (h_pairs[j] >= c->n) return NGIA_ERR_ARG;
  if (count == 0) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return NGIA_OK;
  }
  NGIA_TRY(c->pairs.reserve((size_t)count * 8));
  NGIA_TRY(c->scores.reserve((size_t)count * 4));
  NGIA_CUDA(cudaMemcpyAsync(c->pairs.p, h_pairs, (size_t)count * 8, cudaMemcpyHostToDevice,
                            c->stream));
  NGIA_TRY(ngia::ctx_align_pairs(c, c->pairs.as<uint2>(), count, identity,
                                 c->scores.as<uint32_t>(), stats));
  NGIA_CUDA(cudaMemcpyAsync(h_scores, c->scores.p, (size_t)count * 4, cudaMemcpyDeviceToHost,
                            c->stream));
  NGIA_CUDA(cudaStreamSynchronize(c->stream));
  return NGIA_OK;
}

int ngia_ctx_fast_cluster(ngia_ctx *c, uint32_t identity, uint32_t bands,
                          uint32_t *h_cluster, ngia_stats *stats) {
  if (!c || !h_cluster) return NGIA_ERR_ARG;
  return ngia::ctx_fast_cluster(c, identity, bands, h_cluster, stats);
}

int ngia_ctx_rep_rows(ngia_ctx *c, uint32_t *h_rep, uint32_t bands) {
  if (!c || !h_rep) return NGIA_ERR_ARG;
  if (bands < 1 || bands > c->rep_bands) return NGIA_ERR_ARG;
  NGIA_CUDA(cudaMemcpyAsync(h_rep, c->rep.p, (size_t)bands * c->n * 4,
                            cudaMemcpyDeviceToHost, c->stream));
  NGIA_CUDA(cudaStreamSynchronize(c->stream));
  return NGIA_OK;
}

int ngia_ctx_run_host(ngia_ctx *c, const uint32_t *h_packed, uint64_t packed_words,
                      const uint64_t *h_rec_offsets, const uint32_t *h_lens, uint32_t n,
                      uint32_t identity, uint32_t bands, ngia_edge *h_edges, uint64_t cap,
                      uint64_t *h_n_edges, ngia_stats *stats) {
  if (!c || !h_n_edges) return NGIA_ERR_ARG;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  bool piped = false, sketched = false;
  if (bands >= 1 && bands <= (uint32_t)ngia::kBands)
    NGIA_TRY(ngia::ctx_load_sketch(c, h_packed, packed_words, h_rec_offsets, h_lens, n, &piped,
                                   &sketched));
  if (piped) {
    // no synchronisation until the graph build needs its pair count; the
    // pieced load's code-map check is read after the build
    NGIA_TRY(ngia::ctx_sketch_bucket(c, bands, stats, true, true));
    // the host check of every record, while the device sketches and buckets
    // (nothing launched so far trusts the offsets; the candidates do)
    if (!ngia::records_inside(h_rec_offsets, h_lens, n, packed_words)) {
      cudaStreamSynchronize(c->copy);  // the caller's buffers stay in use until then
      cudaStreamSynchronize(c->layout);
      cudaStreamSynchronize(c->side);
      NGIA_CUDA(cudaStreamSynchronize(c->stream));
      c->n = 0;  // the copies overwrote the resident records: no database until a load
      c->packed_words = 0;
      c->sigs_valid = false;
      c->rep_bands = 0;
      c->n_edges = 0;
      return NGIA_ERR_ARG;
    }
    NGIA_TRY(ngia::ctx_build_graph(c, identity, bands, h_n_edges, stats));
    if (*c->h_flag == 0) {  // the map served every record: the step stands
      if (stats) {
        ngia::ctx_stage_stats(c, stats);
        stats->load_pipelined = 1u;
      }
      return ngia_ctx_edges(c, h_edges, cap);
    }
    if (stats) std::memset(stats, 0, sizeof(*stats));  // start over: the plain load
  }
  NGIA_TRY(ngia::ctx_load(c, h_packed, packed_words, h_rec_offsets, h_lens, n, nullptr, bands));
  NGIA_TRY(ngia::ctx_sketch_bucket(c, bands, stats, false));
  NGIA_TRY(ngia::ctx_build_graph(c, identity, bands, h_n_edges, stats));
  return ngia_ctx_edges(c, h_edges, cap);
}

}  // extern "C"
