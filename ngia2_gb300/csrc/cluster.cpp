// cluster.cpp -- ngia_cluster_file: the `-m clustering` / `-m fast` flow on a
// packed file (src/main.cu:86-156): load the database and its rep rows,
// build the graph on the device, Leiden on the host (or fast greedy
// clustering on the device), then write the result file.
#include <cstdio>
#include <cstring>
#include <vector>

#include "host.hpp"

extern "C" int ngia_cluster_file(const char *packed_path, const char *result_path,
                                 uint32_t identity, uint32_t bands, int fast,
                                 ngia_stats *stats) {
  using namespace ngia;
  if (!packed_path || !result_path) return NGIA_ERR_ARG;
  if (identity < 1 || identity > 99 || bands < 1 || bands > NGIA_BANDS) return NGIA_ERR_ARG;
  ngia_stats local;
  ngia_stats *st = stats ? stats : &local;
  std::memset(st, 0, sizeof(*st));
  ngia_ctx *ctx = nullptr;
  NGIA_TRY_HOST(ngia_ctx_create(&ctx, nullptr));
  int rc = ngia_ctx_load_packed_file(ctx, packed_path, bands, 1);
  PackedDb hdr;
  if (rc == NGIA_OK) rc = read_packed(packed_path, 0, hdr);
  std::vector<uint32_t> cluster;
  if (rc == NGIA_OK) {
    const uint32_t n = hdr.n;
    std::printf("reads count:\t%u\nlongest:\t%u\nshortest:\t%u\n", n, hdr.lens[0],
                hdr.lens[n - 1]);
    cluster.resize(n);
    if (fast) {
      rc = ngia_ctx_fast_cluster(ctx, identity, bands, cluster.data(), st);
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
      if (rc == NGIA_OK) {
        std::printf("compare pairs:\t%llu\n", (unsigned long long)st->candidate_pairs);
        std::printf("unique pairs:\t%llu\nedges:\t%llu\n",
                    (unsigned long long)st->unique_pairs, (unsigned long long)m);
        rc = ngia_leiden(edges.data(), m, n, ngia_leiden_resolution(identity), 42, 1,
                         cluster.data());
      }
    }
  }
  ngia_ctx_destroy(ctx);
  if (rc != NGIA_OK) return rc;
  return ngia_save_result(cluster.data(), (uint32_t)cluster.size(), packed_path, result_path);
}

