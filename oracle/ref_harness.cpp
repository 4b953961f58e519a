/*
 * ref_harness.cpp -- C entry points around the reference's own code, built
 * as a host (OpenMP) library by ref_build.sh from the reference sources with
 * the cuda_stub.h shim.  TEST INFRASTRUCTURE ONLY: tests/ and the reference
 * arm of bench.py call it to obtain the reference's answers and timings.
 * This file is original work; it includes the reference headers, it does not
 * reproduce them.
 */
#include <cstdint>
#include <cstdio>
#include <string>
#include <tuple>
#include <vector>

#include "makedb.hpp"
#include "buildGraph.hpp"
#include "fastClustering.hpp"
#include "leidenParallel.hpp"
#include "saveResult.hpp"

extern "C" {

/* kernel_dynamic (src/buildGraph.hpp:192) over jobs[3*count], in place. */
int ref_align_jobs(const uint32_t *reads, const uint64_t *word_offsets,
                   uint32_t *jobs, uint32_t count, uint32_t identity) {
  const float threshold = identity / 100.0f;
  const size_t *offs = reinterpret_cast<const size_t *>(word_offsets);
  SHIM_LAUNCH(count, BuildGraph::kernel_dynamic, reads, offs, jobs, count,
              threshold);
  return 0;
}

/* makedb (src/main.cu:54-83): index, pack + sketch, group. */
int ref_makedb(const char *fasta, const char *packed) {
  std::vector<MakeDB::seqIndex> idx = MakeDB::makeIndex(fasta);
  if (idx.empty()) return 1;
  size_t n = idx.size();
  if (!MakeDB::packData(fasta, packed, idx)) return 2;
  if (!MakeDB::groupSignatures(packed, n)) return 3;
  return 0;
}

/* makedb without the grouping step: leaves the seq-major signatures. */
int ref_makedb_nogroup(const char *fasta, const char *packed) {
  std::vector<MakeDB::seqIndex> idx = MakeDB::makeIndex(fasta);
  if (idx.empty()) return 1;
  if (!MakeDB::packData(fasta, packed, idx)) return 2;
  return 0;
}

/* readData + buildGraph (src/buildGraph.hpp:125, :256).  Returns the number
 * of edges; the first min(cap, n) edges go to rep/tar/score (score = weight
 * * 100 rounded).  *pairs_out = candidate pairs counted over all bands. */
long ref_build_graph(const char *packed, uint32_t identity, uint32_t bands,
                     int32_t *rep, int32_t *tar, float *weight, long cap) {
  BuildGraph::Data d = BuildGraph::readData(packed, bands);
  if (d.seqCount == 0) return -1;
  bool ok = true;
  std::vector<std::tuple<int, int, float>> g =
      BuildGraph::buildGraph(d, identity, bands, ok);
  BuildGraph::freeMemory(d);
  if (!ok) return -2;
  long m = (long)g.size();
  for (long k = 0; k < m && k < cap; k++) {
    rep[k] = std::get<0>(g[k]);
    tar[k] = std::get<1>(g[k]);
    weight[k] = std::get<2>(g[k]);
  }
  return m;
}

/* LeidenOmp::cluster (src/leidenParallel.hpp:265). */
int ref_leiden(const int32_t *u, const int32_t *v, const float *w, long m,
               int n, float resolution, unsigned seed, int iterations,
               uint32_t *out) {
  std::vector<std::tuple<int, int, float>> e;
  e.reserve((size_t)m);
  for (long k = 0; k < m; k++) e.emplace_back(u[k], v[k], w[k]);
  std::vector<uint32_t> r = LeidenOmp::cluster(e, n, resolution, seed, iterations);
  if ((int)r.size() != n) return -1;
  for (int i = 0; i < n; i++) out[i] = r[i];
  return 0;
}

/* FastClustering::readData + cluster (src/fastClustering.hpp:249). */
int ref_fast_cluster(const char *packed, uint32_t identity, uint32_t bands,
                     uint32_t *out, uint32_t n) {
  FastClustering::Data d = FastClustering::readData(packed, bands);
  if (d.seqCount == 0 || d.seqCount != n) return -1;
  bool ok = true;
  std::vector<uint32_t> r = FastClustering::cluster(d, identity, bands, ok);
  FastClustering::freeMemory(d);
  if (!ok) return -2;
  for (uint32_t i = 0; i < n; i++) out[i] = r[i];
  return 0;
}

/* SaveResult::save (src/saveResult.hpp:31). */
int ref_save(const uint32_t *clusters, uint32_t n, const char *packed,
             const char *result) {
  std::vector<uint32_t> c(clusters, clusters + n);
  SaveResult::save(c, packed, result);
  return 0;
}

}  // extern "C"
