// round.cu -- device buffers and the batched alignment round (round.cuh).
#include "round.cuh"

#include <cstring>
#include <vector>

namespace ngia {

std::atomic<uint64_t> g_alloc_gen{0};

int DevBuf::reserve(size_t want) {
  if (want <= bytes) return NGIA_OK;
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
  ++g_alloc_gen;
  if (want == 0) return NGIA_OK;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    cuda_fail(e);
    return NGIA_ERR_NOMEM;
  }
  bytes = want;
  return NGIA_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

double ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();  // a stage not timed is not an error of the next call
    return 0.0;
  }
  return ms;
}

int instantiate_counted(cudaGraph_t graph, cudaGraphExec_t *exec, uint32_t *kernels) {
  size_t n = 0;
  NGIA_CUDA(cudaGraphGetNodes(graph, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  if (n) NGIA_CUDA(cudaGraphGetNodes(graph, nodes.data(), &n));
  uint32_t k = 0;
  for (size_t i = 0; i < n; ++i) {
    cudaGraphNodeType t;
    NGIA_CUDA(cudaGraphNodeGetType(nodes[i], &t));
    if (t == cudaGraphNodeTypeKernel) ++k;
  }
  NGIA_CUDA(cudaGraphInstantiate(exec, graph, 0));
  note_launches(-(long long)k);
  *kernels = k;
  return NGIA_OK;
}

bool Round::Key::operator==(const Key &o) const {
  return pairs == o.pairs && scores == o.scores && nib == o.nib && packed == o.packed &&
         dplanes == o.dplanes && offs == o.offs && lens == o.lens && m == o.m &&
         identity == o.identity && round_mode == o.round_mode && ab_k == o.ab_k &&
         ab_inv == o.ab_inv && alloc_gen == o.alloc_gen && plan_gen == o.plan_gen;
}

int Round::init(cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  if (s) {
    stream = s;
  } else {
    e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    own_stream_ = e == cudaSuccess;
  }
  for (int k = 0; k < kSide && e == cudaSuccess; ++k) {
    e = cudaStreamCreateWithFlags(&side_[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join_[k], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = cudaEventCreate(&ev_[k]);
  if (e != cudaSuccess) {
    destroy();
    return cuda_fail(e);
  }
  return NGIA_OK;
}

void Round::destroy() {
  if (stream) cudaStreamSynchronize(stream);
  for (int k = 0; k < kSide; ++k) {
    if (side_[k]) {
      cudaStreamSynchronize(side_[k]);
      cudaStreamDestroy(side_[k]);
    }
    if (join_[k]) cudaEventDestroy(join_[k]);
    side_[k] = nullptr;
    join_[k] = nullptr;
  }
  if (fork_) cudaEventDestroy(fork_);
  fork_ = nullptr;
  for (int k = 0; k < 3; ++k) {
    if (ev_[k]) cudaEventDestroy(ev_[k]);
    ev_[k] = nullptr;
  }
  if (exec_) cudaGraphExecDestroy(exec_);
  exec_ = nullptr;
  counters_.release();
  cls_.release();
  cls_sorted_.release();
  order_.release();
  sort_tmp_.release();
  if (own_stream_ && stream) cudaStreamDestroy(stream);
  stream = nullptr;
  own_stream_ = false;
}

int Round::reserve(uint32_t m) {
  const size_t n = m ? m : 1;
  NGIA_TRY(counters_.reserve(sizeof(Counters)));
  NGIA_TRY(cls_.reserve(n * 4));
  NGIA_TRY(cls_sorted_.reserve(n * 4));
  NGIA_TRY(order_.reserve(n * 4));
  NGIA_TRY(sort_tmp_.reserve(radix_sort_scratch_bytes((uint32_t)n, 1)));
  return NGIA_OK;
}

int Round::enqueue(const DbView &db, const uint2 *pairs, uint32_t m, uint32_t identity,
                   uint32_t *scores, cudaEvent_t ev_mid) {
  cudaStream_t s = stream;
  Counters *dc = counters();
  NGIA_CUDA(cudaMemsetAsync(dc, 0, sizeof(Counters), s));
  NGIA_TRY(classify(db.lens, pairs, m, identity, plan, cls_.as<uint32_t>(), dc->class_count,
                    &dc->cells, dc->bounds, s));
  NGIA_TRY(radix_sort_pairs(cls_.as<uint32_t>(), nullptr, cls_sorted_.as<uint32_t>(),
                            order_.as<uint32_t>(), m, 1, 0, kClassKeyBits, sort_tmp_.p, s));
  NGIA_CUDA(cudaMemsetAsync(scores, 0, (size_t)(m ? m : 1) * 4, s));
  if (ev_mid) NGIA_CUDA(cudaEventRecord(ev_mid, s));
  if (m == 0) return NGIA_OK;
  // classes as concurrent branches, widest first (dealt round-robin over the
  // side streams): the few long pairs' warps leave most of the device to the
  // other classes instead of running alone at the end
  int launch_order[kNumClasses - 1];
  launch_order[0] = kGeneralClass;
  for (int c = 1; c < kNumClasses - 1; ++c) launch_order[c] = kGeneralClass - c;
  NGIA_CUDA(cudaEventRecord(fork_, s));
  for (int k = 0; k < kSide; ++k) NGIA_CUDA(cudaStreamWaitEvent(side_[k], fork_, 0));
  int k = 0;
  for (int cl : launch_order) {
    NGIA_TRY(launch_align_class(cl, db.packed, db.nib, db.ab, db.offs, pairs,
                                order_.as<uint32_t>(), dc->bounds, scores, identity, &dc->work,
                                &dc->cursor[cl], side_[k]));
    k = (k + 1) % kSide;
  }
  for (int j = 0; j < kSide; ++j) {
    NGIA_CUDA(cudaEventRecord(join_[j], side_[j]));
    NGIA_CUDA(cudaStreamWaitEvent(s, join_[j], 0));
  }
  return NGIA_OK;
}

int Round::launch(const DbView &db, const uint2 *pairs, uint32_t m, uint32_t identity,
                  uint32_t *scores) {
  NGIA_TRY(reserve(m));
  if (!use_graphs) return enqueue(db, pairs, m, identity, scores, nullptr);
  // everything the captured launches take by value or pointer: the database's
  // buffers and alphabet (a new load may reuse the buffers with another
  // alphabet, whose classes are other kernels), the pairs, the plan
  const Key key{pairs,   scores, db.nib,   db.packed,    db.ab.dplanes, db.offs,
                db.lens, m,      identity, round_mode(), db.ab.K,       db.ab.inv,
                g_alloc_gen.load(), plan_gen};
  if (!exec_ || !(key == key_)) {
    if (exec_) cudaGraphExecDestroy(exec_);
    exec_ = nullptr;
    NGIA_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed));
    int rc = enqueue(db, pairs, m, identity, scores, nullptr);
    cudaGraph_t graph = nullptr;
    const cudaError_t e1 = cudaStreamEndCapture(stream, &graph);
    if (rc == NGIA_OK && e1 != cudaSuccess) rc = cuda_fail(e1);
    if (rc == NGIA_OK) rc = instantiate_counted(graph, &exec_, &exec_kernels_);
    if (graph) cudaGraphDestroy(graph);
    if (rc != NGIA_OK) {
      exec_ = nullptr;
      return rc;
    }
    key_ = key;
  }
  NGIA_CUDA(cudaGraphLaunch(exec_, stream));
  note_launches(exec_kernels_);
  return NGIA_OK;
}

int Round::run(const DbView &db, const uint2 *pairs, uint32_t m, uint32_t identity,
               uint32_t *scores, RoundStats *st) {
  if (st) std::memset(st, 0, sizeof(*st));
  if (m == 0) return NGIA_OK;
  NGIA_TRY(reserve(m));
  NGIA_CUDA(cudaEventRecord(ev_[0], stream));
  if (use_graphs) {
    NGIA_TRY(launch(db, pairs, m, identity, scores));
    NGIA_CUDA(cudaEventRecord(ev_[1], stream));
  } else {
    NGIA_TRY(enqueue(db, pairs, m, identity, scores, ev_[1]));
  }
  NGIA_CUDA(cudaEventRecord(ev_[2], stream));
  NGIA_CUDA(cudaEventSynchronize(ev_[2]));
  if (st) {
    Counters hc;
    NGIA_CUDA(cudaMemcpy(&hc, counters(), sizeof(Counters), cudaMemcpyDeviceToHost));
    st->cells = hc.cells;
    st->work = hc.work;
    if (use_graphs) {
      st->ms_align = ev_ms(ev_[0], ev_[2]);
    } else {
      st->ms_classify = ev_ms(ev_[0], ev_[1]);
      st->ms_align = ev_ms(ev_[1], ev_[2]);
    }
  }
  return NGIA_OK;
}

}  // namespace ngia
