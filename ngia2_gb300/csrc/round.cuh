// round.cuh -- device buffers and the batched alignment round (internal
// header).
//
// A Round owns what one batched alignment needs besides the database and the
// pair list: classification and queue-order scratch, the device counters, a
// stream with side streams for the width classes' concurrent branches, the
// binning plan and a cached CUDA graph of the round.  The context owns one;
// every serving slot owns its own, so that requests run concurrently.
#pragma once

#include <atomic>

#include "align.cuh"
#include "kernels.cuh"

namespace ngia {

// Every device (re)allocation bumps this, so that a captured graph, whose
// nodes hold buffer addresses, is known to be stale.
extern std::atomic<uint64_t> g_alloc_gen;

// Grow-only device buffer.
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  int reserve(size_t want);
  template <typename T>
  T *as() const { return static_cast<T *>(p); }
  void release();
};

struct Counters {  // device-side counters of one graph build or round
  unsigned long long cand_total;
  unsigned long long cells;
  uint64_t unique_total;
  unsigned int class_count[kNumClasses];
  uint32_t fast_count;
  unsigned long long work;  // 32x32 blocks the aligners computed
  unsigned int cursor[kNumClasses];  // pairs taken from each class's queue
  uint32_t bounds[kNumClasses + 1];  // class ranges of the queue order
  unsigned int collect_ticket, collect_error;  // the one-pass candidate collection
};

// The records the aligners read (one index space: offs[i], lens[i]).
struct DbView {
  const uint32_t *packed;  // records with bit planes
  const uint32_t *nib;     // the same records as nibble codes
  Alphabet ab;
  const uint64_t *offs;
  const uint32_t *lens;
};

double ev_ms(cudaEvent_t a, cudaEvent_t b);

// Instantiates a graph captured from a stream.  Its kernel nodes, which their
// launch sites counted while it was captured, are taken back from the launch
// count, and *kernels receives their number for the replays to count.
int instantiate_counted(cudaGraph_t graph, cudaGraphExec_t *exec, uint32_t *kernels);

struct RoundStats {
  unsigned long long cells, work;  // band cells, computed 32x32 blocks
  double ms_classify, ms_align;    // ms_classify is 0 for a graph replay
};

class Round {
 public:
  static constexpr int kSide = 4;
  cudaStream_t stream = nullptr;
  ClassPlan plan = default_plan();
  uint64_t plan_gen = 0;
  bool use_graphs = true;

  // s == nullptr: the round creates its own stream.
  int init(cudaStream_t s);
  void destroy();
  int reserve(uint32_t m);  // scratch for m pairs; never inside a capture
  Counters *counters() const { return counters_.as<Counters>(); }

  // The batched aligner over m device pairs into scores, enqueued on the
  // round's stream with no host round trip: counters zeroed, width classes
  // and their bounds, class-major queue order (longest first), scores
  // zeroed, one persistent launch per class as concurrent branches.  Events
  // ev_start/ev_mid/ev_end (may be null) are recorded around it.
  int enqueue(const DbView &db, const uint2 *pairs, uint32_t m, uint32_t identity,
              uint32_t *scores, cudaEvent_t ev_mid);
  // enqueue through the cached graph when graphs are on (captured on a key
  // change), directly otherwise; then waits and reads the counters.
  int run(const DbView &db, const uint2 *pairs, uint32_t m, uint32_t identity,
          uint32_t *scores, RoundStats *st);
  // Same as run without waiting: the work is only enqueued on `stream`.
  int launch(const DbView &db, const uint2 *pairs, uint32_t m, uint32_t identity,
             uint32_t *scores);

 private:
  DevBuf counters_, cls_, cls_sorted_, order_, sort_tmp_;
  cudaStream_t side_[kSide] = {};
  cudaEvent_t join_[kSide] = {}, fork_ = nullptr, ev_[3] = {};
  bool own_stream_ = false;
  cudaGraphExec_t exec_ = nullptr;
  uint32_t exec_kernels_ = 0;
  struct Key {
    const void *pairs, *scores, *nib, *packed, *dplanes, *offs, *lens;
    uint32_t m, identity;
    int round_mode, ab_k;
    uint64_t ab_inv, alloc_gen, plan_gen;
    bool operator==(const Key &o) const;
  } key_{};
};

}  // namespace ngia
