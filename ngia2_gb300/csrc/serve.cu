// serve.cu -- the serving engine: query batches against a resident database
// (ngia_server_*; the assignment rule and admission are described at the
// declarations in ngia.h).
//
// Index space.  The server keeps one copy of the database records followed by
// one region per slot: record i < N is database record i, records
// N + s * max_queries + j are query j of the request running in slot s.  The
// offsets and lengths arrays follow the same numbering, so a slot's pairs
// (database record, query) go through the batched aligner like any pair of
// the database.
//
// Per request, on the slot's stream: copy in (pinned staging), nibble codes,
// 64-band sketch, per-band lookup of the latest database record with the
// same signature (binary search in the database's sorted signatures), one
// pair slot per (query, band) -- the first band of each distinct candidate
// keeps it, the others are marked empty and skipped by the classifier --,
// the batched round, selection of the first band with a hit, copy out, and a
// host callback that completes the request.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "ctx.cuh"

namespace ngia {

constexpr uint32_t kEmpty = 0xFFFFFFFFu;

// One thread per (query, band): the latest database record (largest index)
// whose band signature equals the query's, or kEmpty.  keys/vals: per band,
// the database's (signature, index) pairs sorted by signature then index.
__global__ void __launch_bounds__(256)
lookup_kernel(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals, uint32_t n,
              const uint32_t *__restrict__ qsigs, uint32_t q, uint32_t *__restrict__ cand) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= q * (uint32_t)kBands) return;
  const uint32_t qi = t / kBands, b = t % kBands;
  const uint32_t s = qsigs[(size_t)b * q + qi];
  const uint32_t *k = keys + (size_t)b * n;
  uint32_t lo = 0, hi = n;  // first position with key > s
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(k + mid) <= s) lo = mid + 1;
    else hi = mid;
  }
  cand[t] = (lo > 0 && __ldg(k + lo - 1) == s) ? __ldg(vals + (size_t)b * n + lo - 1) : kEmpty;
}

// One warp per query: pair slots qi*64 + b.  The first band of each distinct
// candidate keeps a pair (the longer record as rep, the database record on a
// tie); every other slot is empty (x = kEmpty).
__global__ void __launch_bounds__(256)
query_pairs_kernel(const uint32_t *__restrict__ cand, const uint32_t *__restrict__ lens,
                   uint32_t qbase, uint32_t q, uint2 *__restrict__ pairs) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t qi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (qi >= q) return;  // whole warps
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t v0 = cand[qi * kBands + lane], v1 = cand[qi * kBands + 32 + lane];
  const uint32_t m0 = __match_any_sync(kFull, v0), m1 = __match_any_sync(kFull, v1);
  const bool f0 = v0 != kEmpty && (m0 & lt) == 0;
  bool f1 = v1 != kEmpty && (m1 & lt) == 0;
  // a band-(32+l) candidate already seen in bands 0..31 is not new
  for (uint32_t l = 0; l < 32; ++l)
    if (__shfl_sync(kFull, v0, l) == v1) f1 = false;
  const uint32_t g = qbase + qi;
  const uint32_t lq = __ldg(lens + g);
  auto pair_of = [&](uint32_t j) {
    return __ldg(lens + j) >= lq ? make_uint2(j, g) : make_uint2(g, j);
  };
  pairs[qi * kBands + lane] = f0 ? pair_of(v0) : make_uint2(kEmpty, kEmpty);
  pairs[qi * kBands + 32 + lane] = f1 ? pair_of(v1) : make_uint2(kEmpty, kEmpty);
}

// One warp per query: the first band whose pair scored > 0 gives the query
// its candidate's cluster; none: a new cluster.
__global__ void __launch_bounds__(256)
query_select_kernel(const uint2 *__restrict__ pairs, const uint32_t *__restrict__ scores,
                    const uint32_t *__restrict__ cand, const uint32_t *__restrict__ cluster,
                    uint32_t q, uint32_t *__restrict__ out) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t qi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (qi >= q) return;
  const size_t s0 = (size_t)qi * kBands + lane, s1 = s0 + 32;
  const bool h0 = pairs[s0].x != kEmpty && scores[s0] > 0;
  const bool h1 = pairs[s1].x != kEmpty && scores[s1] > 0;
  const uint32_t b0 = __ballot_sync(kFull, h0), b1 = __ballot_sync(kFull, h1);
  if (lane == 0) {
    uint32_t r = NGIA_NEW_CLUSTER;
    if (b0) r = cluster[cand[qi * kBands + __ffs(b0) - 1]];
    else if (b1) r = cluster[cand[qi * kBands + 32 + __ffs(b1) - 1]];
    out[qi] = r;
  }
}

// Plain form: the non-empty pair slots as (rep, tar, 0) jobs, with their slot.
__global__ void __launch_bounds__(256)
compact_jobs_kernel(const uint2 *__restrict__ pairs, uint32_t slots, uint32_t *__restrict__ jobs,
                    uint32_t *__restrict__ where, uint32_t *__restrict__ count) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= slots) return;
  const uint2 p = pairs[k];
  if (p.x == kEmpty) return;
  const uint32_t j = atomicAdd(count, 1u);
  jobs[3 * j] = p.x;
  jobs[3 * j + 1] = p.y;
  jobs[3 * j + 2] = 0;
  where[j] = k;
}

__global__ void __launch_bounds__(256)
scatter_scores_kernel(const uint32_t *__restrict__ jobs, const uint32_t *__restrict__ where,
                      const uint32_t *__restrict__ count, uint32_t *__restrict__ scores) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < *count) scores[where[j]] = jobs[3 * j + 2];
}

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket = 0;
  uint32_t q = 0;
  std::vector<uint32_t> packed, lens, result;
  std::vector<uint64_t> offs;
  size_t bytes = 0;  // working memory while in flight
  Clock::time_point t_submit, t_admit, t_done;
  bool done = false;
  int status = NGIA_OK;
};

struct Server;

struct Slot {
  Server *srv = nullptr;
  int id = 0;
  Round round;                 // its stream runs the slot's requests
  uint64_t word_base = 0;      // first word of the slot's records
  uint32_t index_base = 0;     // N + id * max_queries
  DevBuf sigs, cand, pairs, scores, result, presence, jobs, where, count;
  uint32_t *h_packed = nullptr, *h_lens = nullptr, *h_result = nullptr, *h_count = nullptr;
  uint64_t *h_offs = nullptr;
  Request *req = nullptr;
};

struct Server {
  ngia_server_config cfg{};
  int device = 0;             // the device current at create; every buffer lives there
  uint32_t n = 0;             // database records
  uint64_t db_words = 0;
  Alphabet ab{16, 0};
  uint64_t recode_map = 0;    // nonzero: aligner codes are recoded (dense)
  DevBuf packed, nib, dense, dplanes, offs, lens, keys, vals, cluster;
  std::vector<std::unique_ptr<Slot>> slots;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Request *> queue;
  std::map<uint64_t, std::unique_ptr<Request>> requests;
  uint64_t next_ticket = 1;
  size_t inflight = 0;
  bool stop = false;
  std::thread dispatcher;

  DbView view() const {
    return DbView{packed.as<uint32_t>(), recode_map ? dense.as<uint32_t>() : nib.as<uint32_t>(),
                  ab, offs.as<uint64_t>(), lens.as<uint32_t>()};
  }
};

static void CUDART_CB request_done(void *arg) {
  // host callback (no CUDA calls here): hand the results over, free the slot
  Slot *sl = static_cast<Slot *>(arg);
  Server *s = sl->srv;
  std::lock_guard<std::mutex> lock(s->mu);
  Request *r = sl->req;
  if (r) {
    std::memcpy(r->result.data(), sl->h_result, (size_t)r->q * 4);
    r->t_done = Clock::now();
    r->done = true;
    s->inflight -= r->bytes;
  }
  sl->req = nullptr;
  s->cv.notify_all();
}

// Enqueues one request on a slot's stream; completion arrives through
// request_done.
static int run_request(Server *s, Slot *sl, Request *r) {
  cudaStream_t st = sl->round.stream;
  const uint32_t q = r->q;
  const uint64_t words = r->packed.size();
  std::memcpy(sl->h_packed, r->packed.data(), words * 4);
  for (uint32_t i = 0; i < q; ++i) sl->h_offs[i] = sl->word_base + r->offs[i];
  std::memcpy(sl->h_lens, r->lens.data(), (size_t)q * 4);
  uint32_t *packed = s->packed.as<uint32_t>();
  uint64_t *offs = s->offs.as<uint64_t>() + sl->index_base;
  uint32_t *lens = s->lens.as<uint32_t>() + sl->index_base;
  NGIA_CUDA(cudaMemcpyAsync(packed + sl->word_base, sl->h_packed, words * 4,
                            cudaMemcpyHostToDevice, st));
  NGIA_CUDA(cudaMemcpyAsync(offs, sl->h_offs, (size_t)q * 8, cudaMemcpyHostToDevice, st));
  NGIA_CUDA(cudaMemcpyAsync(lens, sl->h_lens, (size_t)q * 4, cudaMemcpyHostToDevice, st));
  NGIA_TRY(launch_nibbles(packed, offs, lens, q, sl->word_base + s->cfg.max_words,
                          s->nib.as<uint32_t>(), sl->presence.as<uint32_t>(), st));
  if (s->recode_map)
    NGIA_TRY(launch_dense_layouts(packed, offs, q, s->recode_map, s->dense.as<uint32_t>(),
                                  s->dplanes.as<uint32_t>(), st));
  NGIA_TRY(launch_sketch_nibbles(s->nib.as<uint32_t>(), offs, q, sl->sigs.as<uint32_t>(), st));
  const uint32_t slots = q * (uint32_t)kBands;
  lookup_kernel<<<ceil_div(slots, 256u), 256, 0, st>>>(s->keys.as<uint32_t>(),
                                                       s->vals.as<uint32_t>(), s->n,
                                                       sl->sigs.as<uint32_t>(), q,
                                                       sl->cand.as<uint32_t>());
  NGIA_LAUNCHED();
  query_pairs_kernel<<<ceil_div(q * 32u, 256u), 256, 0, st>>>(
      sl->cand.as<uint32_t>(), s->lens.as<uint32_t>(), sl->index_base, q, sl->pairs.as<uint2>());
  NGIA_LAUNCHED();
  uint32_t *scores = sl->scores.as<uint32_t>();
  if (!s->cfg.plain) {
    NGIA_TRY(sl->round.enqueue(s->view(), sl->pairs.as<uint2>(), slots, s->cfg.identity, scores,
                               nullptr));
  } else {
    // the plain form: compact the pairs, one launch of the drop-in kernel
    NGIA_CUDA(cudaMemsetAsync(sl->count.p, 0, 4, st));
    NGIA_CUDA(cudaMemsetAsync(scores, 0, (size_t)slots * 4, st));
    compact_jobs_kernel<<<ceil_div(slots, 256u), 256, 0, st>>>(
        sl->pairs.as<uint2>(), slots, sl->jobs.as<uint32_t>(), sl->where.as<uint32_t>(),
        sl->count.as<uint32_t>());
    NGIA_LAUNCHED();
    NGIA_CUDA(cudaMemcpyAsync(sl->h_count, sl->count.p, 4, cudaMemcpyDeviceToHost, st));
    NGIA_CUDA(cudaStreamSynchronize(st));
    NGIA_TRY(launch_align_jobs(packed, s->offs.as<uint64_t>(), sl->jobs.as<uint32_t>(),
                               *sl->h_count, s->cfg.identity, st));
    scatter_scores_kernel<<<ceil_div(*sl->h_count ? *sl->h_count : 1u, 256u), 256, 0, st>>>(
        sl->jobs.as<uint32_t>(), sl->where.as<uint32_t>(), sl->count.as<uint32_t>(), scores);
    NGIA_LAUNCHED();
  }
  query_select_kernel<<<ceil_div(q * 32u, 256u), 256, 0, st>>>(
      sl->pairs.as<uint2>(), scores, sl->cand.as<uint32_t>(), s->cluster.as<uint32_t>(), q,
      sl->result.as<uint32_t>());
  NGIA_LAUNCHED();
  NGIA_CUDA(cudaMemcpyAsync(sl->h_result, sl->result.p, (size_t)q * 4, cudaMemcpyDeviceToHost,
                            st));
  NGIA_CUDA(cudaLaunchHostFunc(st, request_done, sl));
  return NGIA_OK;
}

// A free slot for a request: slots below small_slots take only small
// requests (a small one takes those first).
static Slot *free_slot(Server *s, bool small) {
  const uint32_t reserved = s->cfg.small_queries ? s->cfg.small_slots : 0u;
  if (small)
    for (uint32_t k = 0; k < reserved && k < s->slots.size(); ++k)
      if (!s->slots[k]->req) return s->slots[k].get();
  for (size_t k = reserved; k < s->slots.size(); ++k)
    if (!s->slots[k]->req) return s->slots[k].get();
  return nullptr;
}

// The request to admit next and its slot: the first small request queued
// (when small requests go first) if a slot takes it, else the front of the
// queue; each within the HBM budget.
static bool next_admission(Server *s, std::deque<Request *>::iterator *which, Slot **slot) {
  auto fits = [&](const Request *r) {
    return s->inflight == 0 || s->inflight + r->bytes <= s->cfg.hbm_budget;
  };
  if (s->cfg.small_queries) {
    for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
      if ((*it)->q > s->cfg.small_queries) continue;
      Slot *sl = free_slot(s, true);
      if (sl && fits(*it)) {
        *which = it;
        *slot = sl;
        return true;
      }
      break;
    }
  }
  const Request *front = s->queue.front();
  Slot *sl = free_slot(s, s->cfg.small_queries && front->q <= s->cfg.small_queries);
  if (sl && fits(front)) {
    *which = s->queue.begin();
    *slot = sl;
    return true;
  }
  return false;
}

static void dispatch_loop(Server *s) {
  // a new thread starts on device 0: make the server's device current before
  // any copy or launch on its streams
  const cudaError_t dev_err = cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    std::deque<Request *>::iterator which;
    Slot *sl = nullptr;
    s->cv.wait(lk, [&] {
      if (s->queue.empty()) return s->stop;
      return next_admission(s, &which, &sl);
    });
    if (s->queue.empty()) break;  // stopping, nothing left to admit
    Request *r = *which;
    s->queue.erase(which);
    sl->req = r;
    s->inflight += r->bytes;
    r->t_admit = Clock::now();
    lk.unlock();
    const int rc = dev_err == cudaSuccess ? run_request(s, sl, r) : cuda_fail(dev_err);
    lk.lock();
    if (rc != NGIA_OK) {  // nothing more was enqueued after the failing call
      lk.unlock();
      cudaStreamSynchronize(sl->round.stream);
      lk.lock();
      r->status = rc;
      r->t_done = Clock::now();
      r->done = true;
      s->inflight -= r->bytes;
      sl->req = nullptr;
      s->cv.notify_all();
    }
  }
}

static size_t request_bytes(uint64_t words, uint32_t q, bool dense) {
  return (size_t)words * 4 * (dense ? 4 : 2) + (size_t)q * (12 + 4 * kBands + 4) +
         (size_t)q * kBands * (4 + 8 + 4 + 12);
}

}  // namespace ngia

struct ngia_server : ngia::Server {};

extern "C" {

static int server_init(ngia_server *s, ngia_ctx *db, const uint32_t *h_cluster,
                       const ngia_server_config *cfg);

int ngia_server_create(ngia_server **out, ngia_ctx *db, const uint32_t *h_cluster,
                       const ngia_server_config *cfg) {
  if (!out || !db || !h_cluster || !cfg) return NGIA_ERR_ARG;
  *out = nullptr;
  if (db->n == 0) return NGIA_ERR_STATE;
  if (cfg->identity < 1 || cfg->identity > 99 || cfg->slots < 1 || cfg->slots > 16 ||
      cfg->max_queries < 1 || cfg->max_words < 1)
    return NGIA_ERR_ARG;
  if (cfg->small_queries && cfg->small_slots >= cfg->slots && !cfg->plain) return NGIA_ERR_ARG;
  ngia_server *s = new (std::nothrow) ngia_server();
  if (!s) return NGIA_ERR_NOMEM;
  const int rc = server_init(s, db, h_cluster, cfg);
  if (rc != NGIA_OK) {
    ngia_server_destroy(s);
    return rc;
  }
  s->dispatcher = std::thread(ngia::dispatch_loop, s);
  *out = s;
  return NGIA_OK;
}

static int server_init(ngia_server *s, ngia_ctx *db, const uint32_t *h_cluster,
                       const ngia_server_config *cfg) {
  using namespace ngia;
  NGIA_CUDA(cudaGetDevice(&s->device));
  if (!db->sigs_valid) NGIA_TRY(ctx_sketch_bucket(db, 1, nullptr));
  s->cfg = *cfg;
  if (s->cfg.plain) {  // one slot, arrival order
    s->cfg.slots = 1;
    s->cfg.small_queries = s->cfg.small_slots = 0;
  }
  if (!s->cfg.small_queries) s->cfg.small_slots = 0;
  const uint32_t n = db->n, S = s->cfg.slots, Q = s->cfg.max_queries;
  const uint64_t W = s->cfg.max_words;
  s->n = n;
  s->db_words = db->packed_words;
  s->ab = db->ab;
  s->recode_map = db->recode_map;
  const uint64_t total_words = db->packed_words + (uint64_t)S * W;
  const uint64_t total_recs = (uint64_t)n + (uint64_t)S * Q;
  if (total_recs > 0xFFFFFFFFull) return NGIA_ERR_ARG;
  cudaStream_t st = db->stream;
  // the database's layouts complete (a pieced load leaves the nibbles out)
  NGIA_TRY(ctx_ready_layouts(db));
  NGIA_TRY(s->packed.reserve(total_words * 4));
  NGIA_TRY(s->nib.reserve(total_words * 4));
  if (s->recode_map) {
    NGIA_TRY(s->dense.reserve(total_words * 4));
    NGIA_TRY(s->dplanes.reserve(total_words * 4));
    s->ab.dplanes = s->dplanes.as<uint32_t>();
  }
  NGIA_TRY(s->offs.reserve(total_recs * 8));
  NGIA_TRY(s->lens.reserve(total_recs * 4));
  NGIA_CUDA(cudaMemcpyAsync(s->packed.p, db->packed.p, db->packed_words * 4,
                            cudaMemcpyDeviceToDevice, st));
  NGIA_CUDA(cudaMemcpyAsync(s->nib.p, db->nib.p, db->packed_words * 4, cudaMemcpyDeviceToDevice,
                            st));
  if (s->recode_map) {
    NGIA_CUDA(cudaMemcpyAsync(s->dense.p, db->nib_dense.p, db->packed_words * 4,
                              cudaMemcpyDeviceToDevice, st));
    NGIA_CUDA(cudaMemcpyAsync(s->dplanes.p, db->dplanes.p, db->packed_words * 4,
                              cudaMemcpyDeviceToDevice, st));
  }
  NGIA_CUDA(cudaMemcpyAsync(s->offs.p, db->offs.p, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
  NGIA_CUDA(cudaMemcpyAsync(s->lens.p, db->lens.p, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
  // per band, the database's (signature, index) sorted by signature then index
  NGIA_TRY(s->keys.reserve((size_t)kBands * n * 4));
  NGIA_TRY(s->vals.reserve((size_t)kBands * n * 4));
  struct Scratch : DevBuf {
    ~Scratch() { release(); }
  } tmp;
  NGIA_TRY(tmp.reserve(radix_sort_scratch_bytes(n, kBands)));
  NGIA_TRY(radix_sort_pairs(db->sigs.as<uint32_t>(), nullptr, s->keys.as<uint32_t>(),
                            s->vals.as<uint32_t>(), n, kBands, 0, 32, tmp.p, st));
  NGIA_TRY(s->cluster.reserve((size_t)n * 4));
  NGIA_CUDA(cudaMemcpyAsync(s->cluster.p, h_cluster, (size_t)n * 4, cudaMemcpyHostToDevice, st));
  NGIA_CUDA(cudaStreamSynchronize(st));
  tmp.release();
  for (uint32_t k = 0; k < S; ++k) {
    s->slots.emplace_back(new (std::nothrow) Slot());
    Slot *sl = s->slots.back().get();
    if (!sl) return NGIA_ERR_NOMEM;
    sl->srv = s;
    sl->id = (int)k;
    sl->word_base = db->packed_words + (uint64_t)k * W;
    sl->index_base = n + k * Q;
    NGIA_TRY(sl->round.init(nullptr));
    sl->round.plan = db->round.plan;
    const size_t slots = (size_t)Q * kBands;
    NGIA_TRY(sl->sigs.reserve(slots * 4));
    NGIA_TRY(sl->cand.reserve(slots * 4));
    NGIA_TRY(sl->pairs.reserve(slots * 8));
    NGIA_TRY(sl->scores.reserve(slots * 4));
    NGIA_TRY(sl->result.reserve((size_t)Q * 4));
    NGIA_TRY(sl->presence.reserve(4));
    NGIA_TRY(sl->round.reserve((uint32_t)slots));
    if (s->cfg.plain) {
      NGIA_TRY(sl->jobs.reserve(slots * 12));
      NGIA_TRY(sl->where.reserve(slots * 4));
      NGIA_TRY(sl->count.reserve(4));
    }
    NGIA_CUDA(cudaMallocHost(&sl->h_packed, W * 4));
    NGIA_CUDA(cudaMallocHost(&sl->h_offs, (size_t)Q * 8));
    NGIA_CUDA(cudaMallocHost(&sl->h_lens, (size_t)Q * 4));
    NGIA_CUDA(cudaMallocHost(&sl->h_result, (size_t)Q * 4));
    NGIA_CUDA(cudaMallocHost(&sl->h_count, 4));
  }
  return NGIA_OK;
}

int ngia_server_submit(ngia_server *s, const uint32_t *h_packed, uint64_t words,
                       const uint64_t *h_offs, const uint32_t *h_lens, uint32_t count,
                       uint64_t *ticket) {
  using namespace ngia;
  if (!s || !ticket || (count && (!h_packed || !h_offs || !h_lens))) return NGIA_ERR_ARG;
  if (count == 0 || count > s->cfg.max_queries || words > s->cfg.max_words) return NGIA_ERR_ARG;
  for (uint32_t i = 0; i < count; ++i) {  // every record inside the words given
    if (h_offs[i] >= words || h_lens[i] > NGIA_MAX_READ) return NGIA_ERR_ARG;
    if (h_offs[i] + 1 + 4ull * ((h_lens[i] + 31) / 32) > words) return NGIA_ERR_ARG;
    if (h_packed[h_offs[i]] != h_lens[i]) return NGIA_ERR_FORMAT;
  }
  std::unique_ptr<Request> r(new (std::nothrow) Request());
  if (!r) return NGIA_ERR_NOMEM;
  r->q = count;
  r->packed.assign(h_packed, h_packed + words);
  r->offs.assign(h_offs, h_offs + count);
  r->lens.assign(h_lens, h_lens + count);
  r->result.assign(count, NGIA_NEW_CLUSTER);
  r->bytes = request_bytes(words, count, s->recode_map != 0);
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->stop) return NGIA_ERR_STATE;
  r->ticket = s->next_ticket++;
  *ticket = r->ticket;
  s->queue.push_back(r.get());
  s->requests[r->ticket] = std::move(r);
  s->cv.notify_all();
  return NGIA_OK;
}

int ngia_server_wait(ngia_server *s, uint64_t ticket, uint32_t *h_cluster,
                     ngia_request_stats *st) {
  using namespace ngia;
  if (!s) return NGIA_ERR_ARG;
  std::unique_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(ticket);
    if (it == s->requests.end()) return NGIA_ERR_ARG;
    Request *p = it->second.get();
    s->cv.wait(lk, [&] { return p->done; });
    r = std::move(it->second);
    s->requests.erase(it);
  }
  if (r->status != NGIA_OK) return r->status;
  if (h_cluster) std::memcpy(h_cluster, r->result.data(), (size_t)r->q * 4);
  if (st) {
    auto ms = [](Clock::time_point a, Clock::time_point b) {
      return std::chrono::duration<double, std::milli>(b - a).count();
    };
    st->queue_ms = ms(r->t_submit, r->t_admit);
    st->run_ms = ms(r->t_admit, r->t_done);
    st->total_ms = ms(r->t_submit, r->t_done);
    st->queries = r->q;
    uint32_t a = 0;
    for (uint32_t v : r->result) a += v != NGIA_NEW_CLUSTER;
    st->assigned = a;
  }
  return NGIA_OK;
}

void ngia_server_destroy(ngia_server *s) {
  if (!s) return;
  // free on the server's device, whatever device the calling thread has current
  int caller_dev = -1;
  if (cudaGetDevice(&caller_dev) != cudaSuccess) caller_dev = -1;
  const bool switched = caller_dev >= 0 && caller_dev != s->device &&
                        cudaSetDevice(s->device) == cudaSuccess;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->dispatcher.joinable()) s->dispatcher.join();
  {  // the requests in flight complete through their callbacks
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv.wait(lk, [&] {
      for (auto &sl : s->slots)
        if (sl && sl->req) return false;
      return true;
    });
  }
  for (auto &sl : s->slots) {
    if (!sl) continue;
    sl->round.destroy();
    if (sl->h_packed) cudaFreeHost(sl->h_packed);
    if (sl->h_offs) cudaFreeHost(sl->h_offs);
    if (sl->h_lens) cudaFreeHost(sl->h_lens);
    if (sl->h_result) cudaFreeHost(sl->h_result);
    if (sl->h_count) cudaFreeHost(sl->h_count);
    ngia::DevBuf *bufs[] = {&sl->sigs,   &sl->cand,     &sl->pairs, &sl->scores, &sl->result,
                            &sl->presence, &sl->jobs,   &sl->where, &sl->count};
    for (ngia::DevBuf *b : bufs) b->release();
  }
  ngia::DevBuf *bufs[] = {&s->packed, &s->nib, &s->dense, &s->dplanes, &s->offs, &s->lens,
                          &s->keys,   &s->vals, &s->cluster};
  for (ngia::DevBuf *b : bufs) b->release();
  delete s;
  if (switched) cudaSetDevice(caller_dev);
}

}  // extern "C"
