// cluster.cpp -- ngia_cluster_file: the `-m clustering` / `-m fast` flow on a
// packed file (src/main.cu:86-156): load the database and its rep rows,
// build the graph on the device, Leiden on the host (or fast greedy
// clustering on the device), then write the result file.  Each phase prints
// its wall time, as the reference's timers do.
#include <cstdio>
#include <cstring>
#include <vector>

#include "host.hpp"

namespace ngia {

int cluster_loaded(ngia_ctx *ctx, const char *packed_path, const char *result_path,
                   uint32_t identity, uint32_t bands, int fast, ngia_stats *st,
                   bool release_device, int device, uint32_t n) {
  PhaseClock timer;
  std::vector<uint32_t> cluster(n);
  std::vector<ngia_edge> edges;
  int rc = NGIA_OK;
  if (fast) {
    rc = ngia_ctx_fast_cluster(ctx, identity, bands, cluster.data(), st);
    timer.lap("fast rounds");
  } else {
    uint64_t m = 0;
    rc = ngia_ctx_build_graph(ctx, identity, bands, &m, st);
    if (rc == NGIA_OK) {
      edges.resize(m);
      rc = ngia_ctx_edges(ctx, edges.data(), m);
    }
    timer.lap("build graph");
  }
  ngia_ctx_destroy(ctx);
  // the device's part is over: a process that owns it releases it while the
  // host clusters and writes
  if (release_device) device_release_start(device);
  if (rc != NGIA_OK) return rc;
  if (fast) {
    size_t roots = 0;
    for (uint32_t i = 0; i < n; ++i) roots += cluster[i] == i;
    std::printf("clusters:\t%zu\n[fast %u rounds]\tfinish\n", roots, bands);
  } else {
    std::printf("compare pairs:\t%llu\n", (unsigned long long)st->candidate_pairs);
    std::printf("unique pairs:\t%llu\nedges:\t%llu\n", (unsigned long long)st->unique_pairs,
                (unsigned long long)edges.size());
    rc = ngia_leiden(edges.data(), edges.size(), n, ngia_leiden_resolution(identity), 42, 1,
                     cluster.data());
    timer.lap("leiden");
    if (rc != NGIA_OK) return rc;
  }
  rc = ngia_save_result(cluster.data(), n, packed_path, result_path);
  timer.lap("save");
  return rc;
}

int cluster_file_run(const char *packed_path, const char *result_path, uint32_t identity,
                     uint32_t bands, int fast, ngia_stats *stats, bool release_device,
                     int device) {
  if (!packed_path || !result_path) return NGIA_ERR_ARG;
  if (identity < 1 || identity > 99 || bands < 1 || bands > NGIA_BANDS) return NGIA_ERR_ARG;
  ngia_stats local;
  ngia_stats *st = stats ? stats : &local;
  std::memset(st, 0, sizeof(*st));
  PhaseClock timer;
  PackedView v;
  int rc = open_packed(packed_path, bands, v);
  timer.lap("read");
  if (rc != NGIA_OK) return rc;
  ngia_ctx *ctx = nullptr;
  NGIA_TRY_HOST(ngia_ctx_create(&ctx, nullptr));
  rc = ngia_ctx_load(ctx, v.packed, v.words, v.offsets.data(), v.lens, v.n, v.rep, bands);
  timer.lap("load");
  if (rc != NGIA_OK) {
    ngia_ctx_destroy(ctx);
    return rc;
  }
  const uint32_t n = v.n;
  std::printf("reads count:\t%u\nlongest:\t%u\nshortest:\t%u\n", n, v.lens[0], v.lens[n - 1]);
  v.f.close_file();
  v.offsets = std::vector<uint64_t>();
  return cluster_loaded(ctx, packed_path, result_path, identity, bands, fast, st,
                        release_device, device, n);
}

}  // namespace ngia

extern "C" int ngia_cluster_file(const char *packed_path, const char *result_path,
                                 uint32_t identity, uint32_t bands, int fast,
                                 ngia_stats *stats) {
  return ngia::cluster_file_run(packed_path, result_path, identity, bands, fast, stats, false,
                                0);
}
