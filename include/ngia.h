/*
 * ngia.h -- C ABI of the GB300 group-then-align library (libngia.so).
 *
 * Drop-in for nGIA2's hot path: minhash sketching, band bucketing, banded
 * bit-parallel LCS alignment and identity-threshold edge emission.  All
 * arithmetic is integer (plus the reference's float threshold tests) and is
 * bit-exact with the reference.
 *
 * Conventions
 *  - Every entry point returns an int status: NGIA_OK (0) or a negative
 *    NGIA_ERR_* code.  Nothing throws across the ABI and nothing prints.
 *  - Pointers named d_* are device pointers owned by the caller; h_* are host
 *    pointers.  `stream` is a cudaStream_t passed as void* (NULL = legacy
 *    default stream).  Calls are asynchronous on `stream` unless documented.
 *  - Entry points that need scratch memory take it from the CUDA stream-ordered
 *    allocator (cudaMallocAsync) on `stream` and release it before returning
 *    control of the stream.
 *  - One host thread per ngia_ctx.  Contexts on different threads are
 *    independent.
 *
 * Data layouts (the reference's packed file, src/makedb.hpp:1-21)
 *  - packed region: records {u32 len; u32 planes[4*ceil(len/32)]}; bit r of
 *    plane e of block b is bit e of the 4-bit code of residue 32*b + r.
 *  - rec_offsets: u64 word offset of each record inside the packed region
 *    (the reference's packedOffsets after src/buildGraph.hpp:172-177).
 *  - signatures / rep rows: band-major u32 [bands][n]; row b of the rep area
 *    is rep[b][i] = largest j < i with sig[b][j] == sig[b][i], else i.
 *  - jobs: u32 triples (rep, tar, score) as kernel_dynamic uses them.
 */
#ifndef NGIA_H
#define NGIA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NGIA_BANDS 64        /* GROUP_BANDS, src/makedb.hpp:45 */
#define NGIA_MAX_READ 65534u /* reads of length >= 0xFFFF are dropped, src/makedb.hpp:118 */

enum {
  NGIA_OK = 0,
  NGIA_ERR_ARG = -1,     /* invalid argument (size, identity, bands, NULL) */
  NGIA_ERR_CUDA = -2,    /* a CUDA runtime call or kernel launch failed */
  NGIA_ERR_NOMEM = -3,   /* device or host allocation failed */
  NGIA_ERR_IO = -4,      /* file could not be read or written completely */
  NGIA_ERR_FORMAT = -5,  /* malformed FASTA or packed file */
  NGIA_ERR_STATE = -6    /* call out of order (e.g. no database loaded) */
};

/* One emitted edge: the reference's tuple<int,int,float>(rep, tar, score/100)
 * (src/buildGraph.hpp:344-347). */
typedef struct ngia_edge {
  int32_t rep;
  int32_t tar;
  float weight;
} ngia_edge;

/* Band-bound rounding of ceil(L - Lt*t) (src/buildGraph.hpp:208-210):
 * NGIA_ROUND_FMA rounds the fused multiply-add once, as a GPU build with
 * multiply-add contraction does; NGIA_ROUND_SPLIT rounds the product first. */
#define NGIA_ROUND_SPLIT 0
#define NGIA_ROUND_FMA 1

const char *ngia_status_string(int status);
/* The cudaError_t of the last NGIA_ERR_CUDA on this thread (0 if none). */
int ngia_last_cuda_error(void);
/* Library version string. */
const char *ngia_version(void);
/* Kernels this process has launched through the library so far. */
unsigned long long ngia_kernel_launches(void);

/* Rounding mode used by the alignment entry points (process-wide; default
 * NGIA_ROUND_FMA).  Returns the previous mode. */
int ngia_set_round_mode(int mode);

/* ---- stage (a): sketch --------------------------------------------------------
 * 64 minhash signatures per record, written band-major: d_sigs[b*n + i].
 * Replaces the signing half of MakeDB::packData (src/makedb.hpp:224-248).
 * No scratch memory. */
int ngia_sketch(const uint32_t *d_packed, const uint64_t *d_rec_offsets,
                uint32_t n, uint32_t *d_sigs, void *stream);

/* ---- stage (b): bucket --------------------------------------------------------
 * Rep rows from band-major signatures: d_rep[b*n + i] for b < bands.
 * Replaces MakeDB::groupSignatures (src/makedb.hpp:289-364): a stable radix
 * sort of (sig, idx) per band and the predecessor chain.  Scratch: about
 * 16 * bands * n bytes from the stream-ordered allocator. */
int ngia_bucket(const uint32_t *d_sigs, uint32_t n, uint32_t bands,
                uint32_t *d_rep, void *stream);

/* Same result as ngia_bucket without allocating anything, for callers that
 * cannot allocate device memory while they run (a plugin in a host program
 * that reserves the device up front, a loop that must never take the
 * allocator's synchronising path, a service whose memory is capped).  No
 * counterpart in the reference, which always allocates.
 * Limit: n * bands <= 1,048,576 (e.g. 16,384 sequences x 64 bands); larger
 * inputs return NGIA_ERR_ARG.  The scratch is a fixed ~16.3 MiB device array
 * that every GPU loading this library holds until the process exits.  The
 * first call on a device looks up that array's device address (make it before
 * any stream capture).  All calls share the array: calls that overlap on the
 * GPU (other streams, other host threads) race and must be serialised by the
 * caller.  Every scratch word is written before it is read, so nothing needs
 * clearing between calls.  The looked-up address is kept per device ordinal;
 * after a reset of the device (cudaDeviceReset) it is looked up again once a
 * call has failed with NGIA_ERR_CUDA, so reset only between calls. */
int ngia_bucket_noalloc(const uint32_t *d_sigs, uint32_t n, uint32_t bands,
                        uint32_t *d_rep, void *stream);

/* ---- stage (c): align ---------------------------------------------------------
 * Drop-in for BuildGraph::kernel_dynamic (src/buildGraph.hpp:192-253, launch
 * at :323; same kernel at src/fastClustering.hpp:183-244, launch at :313):
 * for every job, jobs[3j+2] = identity score of (rep = jobs[3j], tar =
 * jobs[3j+1]); pairs failing the length filter keep their score word.
 * identity in 1..99.  One launch.  No scratch memory. */
int ngia_align_pairs(const uint32_t *d_packed, const uint64_t *d_rec_offsets,
                     uint32_t *d_jobs, uint32_t count, uint32_t identity,
                     void *stream);

/* ---- stage (d): emit ------------------------------------------------------------
 * Edge emission of one job batch (src/buildGraph.hpp:339-349): every job with
 * score > 0 becomes ngia_edge{rep, tar, score/100.0f}, in job order.
 * d_edges needs room for count edges; *d_n_edges (device u32) receives the
 * number written.  Scratch: 4*ceil(count/1024) bytes. */
int ngia_emit_edges(const uint32_t *d_jobs, uint32_t count,
                    ngia_edge *d_edges, uint32_t *d_n_edges, void *stream);

/* Sort + unique of an edge list by (rep, tar, weight), in place on the device
 * (src/buildGraph.hpp:357-358).  *h_n is the count in, the unique count out.
 * Synchronises `stream`.  n_nodes bounds the indices. */
int ngia_sort_unique_edges(ngia_edge *d_edges, uint32_t *h_n, uint32_t n_nodes,
                           void *stream);

/* ---- whole graph build on a resident database -----------------------------------
 * ngia_ctx keeps the packed database, its rep rows and all scratch resident
 * on the device.  Inputs are copied once; every later call reuses them. */
typedef struct ngia_ctx ngia_ctx;

typedef struct ngia_stats {
  uint64_t candidate_pairs; /* pairs over all bands, duplicates included (the
                               reference's "compare pairs", buildGraph.hpp:353) */
  uint64_t unique_pairs;    /* distinct (rep, tar) pairs aligned */
  uint64_t aligned_cells;   /* 1024 x 32x32 blocks visited over unique pairs */
  uint64_t edges;           /* emitted edges (sorted, unique) */
  double ms_sketch, ms_bucket, ms_pairs, ms_align, ms_emit; /* device time */
  uint64_t computed_cells;  /* cells the aligners updated: window words (a
                               little wider than the band) times the column
                               blocks processed before a pair's score was
                               settled (see the early exit in common.cuh) */
  uint32_t load_pipelined;  /* ngia_ctx_run_host: 1 when the upload overlapped
                               the sketch (ms_sketch then spans both) */
} ngia_stats;

int ngia_ctx_create(ngia_ctx **ctx, void *stream);
void ngia_ctx_destroy(ngia_ctx *ctx);

/* Load a database from host arrays: the packed region (words), record
 * offsets, read lengths (index order) and optionally `bands` rep rows
 * (band-major; NULL = compute them on the device with sketch + bucket).
 * The records are trusted as a packed file's are: record i starts at word
 * h_rec_offsets[i] with its length word equal to h_lens[i], and its
 * 1 + 4*ceil(len/32) words end inside the region (makedb's files and
 * ngia_pack_records' output are so; ngia_ctx_load_packed_file checks the
 * offsets against the read lengths, not the length words).  The same holds
 * for ngia_ctx_run_host and ngia_stream_graph. */
int ngia_ctx_load(ngia_ctx *ctx, const uint32_t *h_packed, uint64_t packed_words,
                  const uint64_t *h_rec_offsets, const uint32_t *h_lens,
                  uint32_t n, const uint32_t *h_rep, uint32_t bands);

/* Same from a packed file written by makedb (reference format). */
int ngia_ctx_load_packed_file(ngia_ctx *ctx, const char *path, uint32_t bands,
                              int use_file_rep_rows);

/* Recompute sketches and rep rows on the device from the loaded planes. */
int ngia_ctx_sketch_bucket(ngia_ctx *ctx, uint32_t bands);

/* buildGraph: candidates of bands 0..bands-1, deduplicated, aligned
 * (length-binned batched kernels), emitted, sorted and uniqued on the device.
 * Result stays on the device; *h_n_edges receives the count.  Synchronises. */
int ngia_ctx_build_graph(ngia_ctx *ctx, uint32_t identity, uint32_t bands,
                         uint64_t *h_n_edges, ngia_stats *stats);

/* One device's share of ngia_ctx_build_graph when the graph of one database
 * is built by `parts` devices (each holding the database): the distinct
 * candidate pairs, in the order the collection writes them, are cut into
 * `parts` contiguous ranges of about equal band cells (the reference's 32x32
 * blocks, src/buildGraph.hpp:208-217), and this call aligns and emits range
 * `part` only.  h_range (optional) receives the range's [first, end); the
 * edges stay on the device (ngia_ctx_edges), sorted and unique.  The union of
 * all parts' edges, sorted by (rep, tar), is ngia_ctx_build_graph's edge list:
 * the exchange is one gather of the compacted edges before the host's sort and
 * Leiden.  The reference runs on one device (src/buildGraph.hpp:101-102).
 * Synchronises. */
int ngia_ctx_build_graph_part(ngia_ctx *ctx, uint32_t identity, uint32_t bands, uint32_t part,
                              uint32_t parts, uint64_t *h_range, uint64_t *h_n_edges,
                              ngia_stats *stats);

/* The whole device hot path on the resident planes: sketch + bucket of
 * `bands` rep rows, then ngia_ctx_build_graph.  Fills every stats field.
 * Synchronises. */
int ngia_ctx_group_align(ngia_ctx *ctx, uint32_t identity, uint32_t bands,
                         uint64_t *h_n_edges, ngia_stats *stats);

/* A check of the candidate collection's bounded wait (the decoupled look-back
 * of ngia_ctx_build_graph, in which each block of targets waits for the
 * earlier blocks' counts): runs the collection with its ticket counter
 * started at 1, so the first block's count is never published and every
 * block gives up after spin_limit polls (1 .. 2^22).  Returns NGIA_ERR_CUDA,
 * the error the graph build reports when a wait gives up, and leaves the
 * context usable; NGIA_OK would mean a wait did not give up.  Testing aid,
 * no counterpart in the reference.  Synchronises. */
int ngia_ctx_test_lookback_timeout(ngia_ctx *ctx, uint32_t identity, uint32_t bands,
                                   uint32_t spin_limit);

/* Copy the last graph's edges to the host (cap entries at most). */
int ngia_ctx_edges(ngia_ctx *ctx, ngia_edge *h_edges, uint64_t cap);

/* Batched alignment of caller-given pairs on the resident database: the same
 * scores as ngia_align_pairs (the kernel_dynamic contract, src/buildGraph.hpp
 * :192-253; 0 for pairs failing the length filter), computed by the
 * length-binned persistent kernels: pairs are binned by band width, each bin
 * is queued longest first and taken by a persistent grid -- one pair per lane
 * for narrow bands, one pair per group of 8, 16 or 32 lanes for wide ones.
 * d_pairs: count (rep, tar) u32 index pairs on the device, every index below
 * the loaded record count (not checked); d_scores: count u32 out.  The
 * context's own pair scratch is not touched.  Synchronises. */
int ngia_ctx_align_pairs(ngia_ctx *ctx, const uint32_t *d_pairs, uint32_t count,
                         uint32_t identity, uint32_t *d_scores, ngia_stats *stats);

/* How the batched aligner bins pairs (what ngia_ctx_autotune picks).  Width
 * classes: one pair per lane with a window of W = 4, 5, ..., 12, 14, 16 words for
 * pairs whose window ls + min(rs, nr) (in 32-residue blocks) is at most
 * stream_max; otherwise the first group class -- G lanes per pair with K
 * words per lane: (8,3) (8,4) (16,4) (16,6) (32,4) (32,6) (32,8) (32,16) -- whose
 * group_limit admits the band (ls + rs <= group_limit, or a rep of at most G
 * slices); otherwise one pair per thread.  group_limit 0 leaves a class
 * unused; a limit above (G-1)K + G is refused.  Scores never depend on the
 * plan. */
#define NGIA_GROUP_CLASSES 8
typedef struct ngia_plan {
  uint32_t stream_max; /* 4..16 */
  uint32_t group_limit[NGIA_GROUP_CLASSES];
} ngia_plan;

int ngia_ctx_get_plan(ngia_ctx *ctx, ngia_plan *plan);
int ngia_ctx_set_plan(ngia_ctx *ctx, const ngia_plan *plan);

/* Times the batched round on the given device pairs (reps runs per
 * candidate, the best kept) for plans around the current one -- the widest
 * one-pair-per-lane window and each group class on or off -- by coordinate
 * descent, and keeps the fastest as the context's plan.  *best_ms receives
 * its time.  Synchronises. */
int ngia_ctx_autotune(ngia_ctx *ctx, const uint32_t *d_pairs, uint32_t count,
                      uint32_t identity, int reps, ngia_plan *best, double *best_ms);

/* Whether ngia_ctx_align_pairs captures its round (classification, queue
 * sort and every class launch) as a CUDA graph and replays it while the
 * pair/score addresses, count, identity, rounding, plan and the loaded
 * database (its buffers and alphabet) stay the same, and whether the
 * bucketing of every graph build is replayed the same way while its buffers,
 * record count and bands stay the same (default on).  Returns the previous
 * setting (0/1), or NGIA_ERR_ARG. */
int ngia_ctx_use_graphs(ngia_ctx *ctx, int on);

/* Same from host arrays (indices checked, NGIA_ERR_ARG when one is out of
 * range); uses the context's pair buffers. */
int ngia_ctx_align_pairs_host(ngia_ctx *ctx, const uint32_t *h_pairs, uint32_t count,
                              uint32_t identity, uint32_t *h_scores, ngia_stats *stats);

/* ---- packing on the device ----------------------------------------------------------
 * Residues (ASCII, one byte each, record i at d_starts[i], d_lens[i] bytes)
 * into packed records at word offsets d_rec_offsets[i]: [u32 L][4*ceil(L/32)
 * plane words], codes from the reduced 15-letter table -- the packing half of
 * MakeDB::packData (src/makedb.hpp:162-171,223-231).  One warp per record,
 * plane words from ballots.  The records must not overlap. */
int ngia_pack(const uint8_t *d_residues, const uint64_t *d_starts, const uint32_t *d_lens,
              uint32_t n, const uint64_t *d_rec_offsets, uint32_t *d_packed, void *stream);

/* Same from host arrays, records placed back to back: h_rec_offsets receives
 * each record's word offset; h_packed needs room for sum(1 + 4*ceil(L/32))
 * words (`words`).  Allocates its device buffers; synchronous. */
int ngia_pack_records(const uint8_t *h_residues, uint64_t residue_bytes,
                      const uint64_t *h_starts, const uint32_t *h_lens, uint32_t n,
                      uint32_t *h_packed, uint64_t words, uint64_t *h_rec_offsets);

/* ---- a database larger than device memory ----------------------------------------
 * The graph build of ngia_ctx_group_align (sketch + bucket of `bands` rows,
 * candidates, batched alignment, sorted unique edges) for records held in
 * host memory, streamed through at most `chunk_bytes` of device memory for
 * records (three chunk slots of planes, nibble codes -- recoded ones while
 * aligning -- and code planes; the
 * rest -- signatures, rep rows, lengths, offsets, pairs, scores -- grows with
 * the record count only and stays on the device).  The records pass through
 * pinned double-buffered copies twice: once to sketch them, once per block
 * of pairs (rep chunk, target chunk) to align them; records that are
 * themselves page-locked (cudaHostAlloc'd or registered) and span at most
 * 4 GiB are copied from in place instead.  The edges equal the
 * resident path's.  Records must be in index order (increasing offsets, not
 * overlapping); h_edges needs room for the edges (NGIA_ERR_NOMEM if cap is
 * too small).  Replaces the reference's managed-memory oversubscription
 * (src/buildGraph.hpp:58-65,143-171). */
typedef struct ngia_stream_stats {
  uint64_t chunks, chunk_loads, bytes_h2d_sketch, bytes_h2d_align;
  uint64_t candidate_pairs, unique_pairs, aligned_cells, computed_cells, edges;
  double ms_sketch, ms_bucket, ms_pairs, ms_align, ms_emit, ms_total;
} ngia_stream_stats;

int ngia_stream_graph(const uint32_t *h_packed, uint64_t words, const uint64_t *h_offs,
                      const uint32_t *h_lens, uint32_t n, uint32_t identity, uint32_t bands,
                      uint64_t chunk_bytes, ngia_edge *h_edges, uint64_t cap,
                      uint64_t *n_edges, ngia_stream_stats *stats);

/* ---- serving: query batches against a resident database ------------------------
 * A server holds a database (a loaded context's records, copied, with their
 * 64-band signatures sorted per band and the database's cluster ids) and
 * assigns query sequences to its clusters at one identity, by fast mode's
 * rule (src/fastClustering.hpp:249-352) against the database snapshot: in
 * band order 0..63, a query's candidate in a band is the latest database
 * record (in index order) with the same band signature; the pair is aligned
 * with the longer record as rep (the database record on a tie), and the first
 * band whose candidate scores > 0 gives the query that record's cluster id; a
 * query with no hit opens a new cluster (NGIA_NEW_CLUSTER).  Queries never
 * see each other, so a result does not depend on what else is in flight.
 *
 * Requests (batches of queries as packed records) are admitted in arrival
 * order (or small ones first, see ngia_server_config) while a slot is free
 * and the working bytes of the requests in flight stay within the HBM budget
 * (a request larger than the budget runs alone).
 * Each slot runs its request -- copy in, sketch, signature lookup, batched
 * alignment, selection, copy out -- on its own stream, so requests overlap on
 * the device.  plain = 1 gives the per-request plain form to compare with: one
 * slot, and the one-thread-per-pair drop-in kernel over the request's pairs.
 * A server belongs to the device current when it is created: its dispatcher
 * thread makes that device current, and destroy frees on it. */
#define NGIA_NEW_CLUSTER 0xFFFFFFFFu
typedef struct ngia_server ngia_server;
typedef struct ngia_server_config {
  uint32_t identity;    /* 1..99 */
  uint32_t slots;       /* requests in flight at once, 1..16 */
  uint32_t max_queries; /* per request */
  uint64_t max_words;   /* packed-record words per request */
  uint64_t hbm_budget;  /* bytes of request working memory in flight */
  int plain;
  /* Admission order.  small_queries = 0: arrival order, any free slot.  Else
   * a request of at most small_queries queries is admitted ahead of the
   * larger ones queued before it, and slots 0..small_slots-1 take only such
   * requests, so small requests never wait behind large ones for a slot
   * (small_slots < slots). */
  uint32_t small_queries;
  uint32_t small_slots;
} ngia_server_config;
typedef struct ngia_request_stats {
  double queue_ms, run_ms, total_ms; /* submit->admit, admit->done, submit->done */
  uint32_t queries, assigned;        /* assigned: queries given an existing cluster */
} ngia_request_stats;

/* db: a loaded context (its records are copied; it may be destroyed after).
 * h_cluster: the database's cluster id per record (e.g. from
 * ngia_ctx_fast_cluster).  Computes the context's signatures if needed. */
int ngia_server_create(ngia_server **srv, ngia_ctx *db, const uint32_t *h_cluster,
                       const ngia_server_config *cfg);
/* Queues a request (the arrays are copied before return): count packed
 * records (h_offs: word offset of each in h_packed, h_lens: lengths).  Each
 * record is checked: inside the words given (else NGIA_ERR_ARG), its length
 * word equal to h_lens[i] (else NGIA_ERR_FORMAT). */
int ngia_server_submit(ngia_server *srv, const uint32_t *h_packed, uint64_t words,
                       const uint64_t *h_offs, const uint32_t *h_lens, uint32_t count,
                       uint64_t *ticket);
/* Waits for a request; h_cluster receives a cluster id (or NGIA_NEW_CLUSTER)
 * per query.  The ticket is spent. */
int ngia_server_wait(ngia_server *srv, uint64_t ticket, uint32_t *h_cluster,
                     ngia_request_stats *stats);
/* Finishes the requests in flight and queued, then frees everything. */
void ngia_server_destroy(ngia_server *srv);

/* Fast greedy clustering (src/fastClustering.hpp:249-352): per band, targets
 * not yet assigned are aligned against their rep and assigned on a hit;
 * h_cluster[i] = root index.  Synchronises. */
int ngia_ctx_fast_cluster(ngia_ctx *ctx, uint32_t identity, uint32_t bands,
                          uint32_t *h_cluster, ngia_stats *stats);

/* The loaded records' 64 signatures, band-major [64][n], after
 * ngia_ctx_sketch_bucket (NGIA_ERR_STATE before). */
int ngia_ctx_sigs(ngia_ctx *ctx, uint32_t *h_sigs);

/* For a database of at most four residue codes (nucleotides), the sketch reads
 * part of the band hashes of each 8-mer from a table of all 4^8 8-mers (the
 * same signatures; a table row gather for those bands instead of hashing).
 * On by default; returns the previous setting (0/1). */
int ngia_ctx_use_sketch_table(ngia_ctx *ctx, int on);
/* 1 when the context's sketch goes through that table (on, and the loaded
 * database qualifies), else 0. */
int ngia_ctx_sketch_table_active(ngia_ctx *ctx);
/* How many of the 64 bands that table holds (the rest are hashed meanwhile:
 * the table's row gathers load L2 while the hashes load the logic pipe). */
int ngia_sketch_table_bands(void);

/* Copy the device rep rows (bands x n) to the host. */
int ngia_ctx_rep_rows(ngia_ctx *ctx, uint32_t *h_rep, uint32_t bands);

/* End-to-end call on host buffers: copy the database in, sketch + bucket,
 * build the graph, copy the edges out (the reference's makedb grouping plus
 * buildGraph in one call).  Device buffers of the context are reused across
 * calls.  When the previous load's residue codes took the table sketch (four
 * codes or fewer, none 0), the upload goes in pieces that are sketched as they
 * land, under that code map; a database whose codes fall outside it, or whose
 * record offsets are not in order, is loaded the plain way (same result;
 * stats->load_pipelined tells which).  Pinned host buffers give the upload
 * the link's full bandwidth.  Records outside the region (see ngia_ctx_load)
 * are refused with NGIA_ERR_ARG; the pieced upload checks them on the host
 * while the device already copies, lays out, sketches and buckets (kernels
 * that bound every record by the region), so after that refusal the context
 * holds no database until the next load.  Synchronises. */
int ngia_ctx_run_host(ngia_ctx *ctx, const uint32_t *h_packed,
                      uint64_t packed_words, const uint64_t *h_rec_offsets,
                      const uint32_t *h_lens, uint32_t n, uint32_t identity,
                      uint32_t bands, ngia_edge *h_edges, uint64_t cap,
                      uint64_t *h_n_edges, ngia_stats *stats);

/* Measured throughput of 32-bit three-input logic ops (lop3) over the whole
 * device, in lane-operations per second: the integer-ALU ceiling used as the
 * roofline of the integer-bound kernels.  Synchronises. */
int ngia_int32_peak(void *stream, double *ops_per_s);

/* ---- host side of the drop-in (C++ host code in the same library) -------------- */

/* makedb (src/main.cu:54-83): FASTA -> packed file.  Index, length filter and
 * stable length-descending order on the host, pack on the host, sketch and
 * bucket on the device.  Returns the number of sequences in *n_out. */
int ngia_makedb(const char *fasta_path, const char *packed_path, uint32_t *n_out);

/* LeidenOmp::cluster (src/leidenParallel.hpp:265-322) on the host. */
int ngia_leiden(const ngia_edge *h_edges, uint64_t m, uint32_t n,
                float resolution, uint32_t seed, int iterations,
                uint32_t *h_cluster);

/* The resolution main() derives from the identity (src/main.cu:114-116). */
float ngia_leiden_resolution(uint32_t identity);

/* SaveResult::save (src/saveResult.hpp:31-83). */
int ngia_save_result(const uint32_t *h_cluster, uint32_t n,
                     const char *packed_path, const char *result_path);

/* The whole `-m clustering` / `-m fast` mode on a packed file
 * (src/main.cu:86-156).  fast != 0 selects fast mode. */
int ngia_cluster_file(const char *packed_path, const char *result_path,
                      uint32_t identity, uint32_t bands, int fast,
                      ngia_stats *stats);

#ifdef __cplusplus
}
#endif
#endif
