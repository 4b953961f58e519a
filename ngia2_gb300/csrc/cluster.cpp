// cluster.cpp -- ngia_cluster_file: the `-m clustering` / `-m fast` flow on a
// packed file (src/main.cu:86-156): load the database and its rep rows,
// build the graph on the device, Leiden on the host (or fast greedy
// clustering on the device), then write the result file.  Each phase prints
// its wall time, as the reference's timers do.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <vector>

#include "host.hpp"

namespace {

struct PhaseTimer {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  void lap(const char *what) {
    const auto t1 = std::chrono::steady_clock::now();
    std::printf("  [%s]\t%.6f s\n", what, std::chrono::duration<double>(t1 - t0).count());
    t0 = t1;
  }
};

}  // namespace

extern "C" int ngia_cluster_file(const char *packed_path, const char *result_path,
                                 uint32_t identity, uint32_t bands, int fast,
                                 ngia_stats *stats) {
  using namespace ngia;
  if (!packed_path || !result_path) return NGIA_ERR_ARG;
  if (identity < 1 || identity > 99 || bands < 1 || bands > NGIA_BANDS) return NGIA_ERR_ARG;
  ngia_stats local;
  ngia_stats *st = stats ? stats : &local;
  std::memset(st, 0, sizeof(*st));
  PhaseTimer timer;
  ngia_ctx *ctx = nullptr;
  NGIA_TRY_HOST(ngia_ctx_create(&ctx, nullptr));
  timer.lap("device init");
  PackedDb db;
  int rc = read_packed(packed_path, bands, db);
  if (rc == NGIA_OK)
    rc = ngia_ctx_load(ctx, db.packed.data(), db.packed.size(), db.offsets.data(),
                       db.lens.data(), db.n, db.rep.data(), bands);
  timer.lap("load");
  std::vector<uint32_t> cluster;
  if (rc == NGIA_OK) {
    const uint32_t n = db.n;
    std::printf("reads count:\t%u\nlongest:\t%u\nshortest:\t%u\n", n, db.lens[0],
                db.lens[n - 1]);
    cluster.resize(n);
    if (fast) {
      rc = ngia_ctx_fast_cluster(ctx, identity, bands, cluster.data(), st);
      timer.lap("fast rounds");
      if (rc == NGIA_OK) {
        size_t roots = 0;
        for (uint32_t i = 0; i < n; ++i) roots += cluster[i] == i;
        std::printf("clusters:\t%zu\n[fast %u rounds]\tfinish\n", roots, bands);
      }
    } else {
      uint64_t m = 0;
      rc = ngia_ctx_build_graph(ctx, identity, bands, &m, st);
      std::vector<ngia_edge> edges(m);
      if (rc == NGIA_OK) rc = ngia_ctx_edges(ctx, edges.data(), m);
      timer.lap("build graph");
      if (rc == NGIA_OK) {
        std::printf("compare pairs:\t%llu\n", (unsigned long long)st->candidate_pairs);
        std::printf("unique pairs:\t%llu\nedges:\t%llu\n",
                    (unsigned long long)st->unique_pairs, (unsigned long long)m);
        rc = ngia_leiden(edges.data(), m, n, ngia_leiden_resolution(identity), 42, 1,
                         cluster.data());
        timer.lap("leiden");
      }
    }
  }
  ngia_ctx_destroy(ctx);
  db = PackedDb();
  if (rc != NGIA_OK) return rc;
  rc = ngia_save_result(cluster.data(), (uint32_t)cluster.size(), packed_path, result_path);
  timer.lap("save");
  return rc;
}
