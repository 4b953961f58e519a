// leiden.cpp -- community detection on the host, unchanged in behaviour from
// LeidenOmp::cluster (src/leidenParallel.hpp:36-324), so that the clusters are
// bit-exact with the reference for the same edge set, seed and iterations.
//
// The algorithm (RB-configuration quality, unweighted undirected graph):
//   repeat over at most 32 aggregation levels:
//     local moving  -- sequential sweeps over nodes in index order; a node
//                      moves to the neighbouring community of largest strictly
//                      positive gain  w_c - g*k*(K_c + k)/M - (w_old - g*k*K_old/M)
//                      (first maximum in neighbour order), at most 300 sweeps;
//     refinement    -- nodes in a Fisher-Yates order from mt19937_64; a
//                      singleton sub-community joins a random sub-community of
//                      a same-community neighbour when the gain is >= 0;
//     aggregation   -- collapse the refined partition into a weighted graph;
//   then number the top-level communities by first occurrence in index order.
// Edge weights are integer counts, so every weight sum is exact; the gain
// expressions are evaluated in the reference's operand order (this file is
// compiled with -ffp-contract=off).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <utility>
#include <vector>

#include "host.hpp"

namespace ngia {

namespace {

struct Graph {
  int n = 0;
  std::vector<int> row, adj;
  std::vector<double> awt, deg;
  double total = 0.0;
};

// Adjacency from an edge list already normalised (u <= v), sorted and unique.
Graph graph_from_sorted(int n, const std::vector<int> &from, const std::vector<int> &to,
                        const std::vector<double> &wt) {
  Graph g;
  g.n = n;
  const size_t m = from.size();
  g.row.assign((size_t)n + 1, 0);
  for (size_t e = 0; e < m; ++e) {
    g.row[(size_t)from[e] + 1]++;
    g.row[(size_t)to[e] + 1]++;
  }
  for (int v = 0; v < n; ++v) g.row[(size_t)v + 1] += g.row[(size_t)v];
  g.adj.resize(2 * m);
  g.awt.resize(2 * m);
  std::vector<int> fill(g.row.begin(), g.row.end() - 1);
  for (size_t e = 0; e < m; ++e) {
    const int u = from[e], v = to[e];
    const double w = wt[e];
    g.adj[(size_t)fill[(size_t)u]] = v;
    g.awt[(size_t)fill[(size_t)u]++] = w;
    g.adj[(size_t)fill[(size_t)v]] = u;
    g.awt[(size_t)fill[(size_t)v]++] = w;
  }
  g.deg.assign((size_t)n, 0.0);
  for (int v = 0; v < n; ++v) {
    double s = 0.0;
    for (int k = g.row[(size_t)v]; k < g.row[(size_t)v + 1]; ++k) s += g.awt[(size_t)k];
    g.deg[(size_t)v] = s;
  }
  g.total = std::accumulate(g.deg.begin(), g.deg.end(), 0.0);
  return g;
}

typedef std::pair<std::pair<int, int>, double> WEdge;

// Sort weighted (u <= v) edges and merge duplicates by summing weights.
Graph graph_from_edges(int n, std::vector<WEdge> &es) {
  std::sort(es.begin(), es.end());
  std::vector<int> from, to;
  std::vector<double> wt;
  for (size_t i = 0; i < es.size();) {
    size_t j = i;
    double s = 0.0;
    while (j < es.size() && es[j].first == es[i].first) s += es[j++].second;
    from.push_back(es[i].first.first);
    to.push_back(es[i].first.second);
    wt.push_back(s);
    i = j;
  }
  return graph_from_sorted(n, from, to, wt);
}

// Communities of v's neighbours (self loops skipped) with summed weights, in
// order of first appearance in v's adjacency.
void neighbour_communities(const Graph &g, const std::vector<int> &memb, int v,
                           std::vector<int> &comm, std::vector<double> &w) {
  comm.clear();
  w.clear();
  for (int k = g.row[(size_t)v]; k < g.row[(size_t)v + 1]; ++k) {
    const int u = g.adj[(size_t)k];
    if (u == v) continue;
    const int c = memb[(size_t)u];
    size_t i = 0;
    while (i < comm.size() && comm[i] != c) ++i;
    if (i < comm.size()) {
      w[i] += g.awt[(size_t)k];
    } else {
      comm.push_back(c);
      w.push_back(g.awt[(size_t)k]);
    }
  }
}

int local_moving(const Graph &g, std::vector<int> &memb, std::vector<double> &tot,
                 double gamma) {
  const double M = g.total;
  if (M <= 0.0) return 0;
  int moves_total = 0;
  std::vector<int> comm;
  std::vector<double> w;
  for (int sweep = 0; sweep < 300; ++sweep) {
    int moves = 0;
    for (int v = 0; v < g.n; ++v) {
      if (g.row[(size_t)v] == g.row[(size_t)v + 1]) continue;
      const int old = memb[(size_t)v];
      const double k = g.deg[(size_t)v];
      neighbour_communities(g, memb, v, comm, w);
      double w_old = 0.0;
      for (size_t i = 0; i < comm.size(); ++i)
        if (comm[i] == old) w_old = w[i];
      int best = old;
      double best_gain = 0.0;
      for (size_t i = 0; i < comm.size(); ++i) {
        const int c = comm[i];
        if (c == old) continue;
        const double gain = (w[i] - gamma * k * (tot[(size_t)c] + k) / M) -
                            (w_old - gamma * k * tot[(size_t)old] / M);
        if (gain > best_gain) {
          best_gain = gain;
          best = c;
        }
      }
      if (best != old && best_gain > 0.0) {
        memb[(size_t)v] = best;
        tot[(size_t)old] -= k;
        tot[(size_t)best] += k;
        ++moves;
      }
    }
    moves_total += moves;
    if (moves == 0) break;
  }
  return moves_total;
}

// Refinement inside the coarse partition; returns the number of
// sub-communities and renumbers `sub` by first occurrence.
int refine(const Graph &g, const std::vector<int> &coarse, std::vector<int> &sub,
           double gamma, uint64_t seed) {
  const int n = g.n;
  const double M = g.total;
  sub.resize((size_t)n);
  std::vector<double> stot((size_t)n);
  std::vector<int> size((size_t)n, 1);
  for (int v = 0; v < n; ++v) {
    sub[(size_t)v] = v;
    stot[(size_t)v] = g.deg[(size_t)v];
  }
  std::vector<int> order((size_t)n);
  std::iota(order.begin(), order.end(), 0);
  std::mt19937_64 rng(seed);
  for (size_t i = order.size() - 1; i > 0; --i) {
    const size_t j = (size_t)(rng() % (i + 1));
    std::swap(order[i], order[j]);
  }
  std::vector<int> cand;
  for (int v : order) {
    const int sc = sub[(size_t)v];
    if (size[(size_t)sc] != 1) continue;
    const int cc = coarse[(size_t)v];
    cand.clear();
    for (int k = g.row[(size_t)v]; k < g.row[(size_t)v + 1]; ++k) {
      const int u = g.adj[(size_t)k];
      if (u == v || coarse[(size_t)u] != cc) continue;
      const int s2 = sub[(size_t)u];
      if (std::find(cand.begin(), cand.end(), s2) == cand.end()) cand.push_back(s2);
    }
    if (cand.empty()) continue;
    const int target = cand[(size_t)(rng() % cand.size())];
    if (target == sc) continue;
    double w_old = 0.0, w_new = 0.0;
    for (int k = g.row[(size_t)v]; k < g.row[(size_t)v + 1]; ++k) {
      const int u = g.adj[(size_t)k];
      if (u == v) continue;
      const int s2 = sub[(size_t)u];
      if (s2 == sc) w_old += g.awt[(size_t)k];
      if (s2 == target) w_new += g.awt[(size_t)k];
    }
    const double kv = g.deg[(size_t)v];
    const double gain = (w_new - gamma * kv * (stot[(size_t)target] + kv) / M) -
                        (w_old - gamma * kv * stot[(size_t)sc] / M);
    if (gain >= 0) {
      sub[(size_t)v] = target;
      stot[(size_t)sc] -= g.deg[(size_t)v];
      stot[(size_t)target] += g.deg[(size_t)v];
      size[(size_t)sc] = 0;
      size[(size_t)target] += 1;
    }
  }
  std::vector<int> renum((size_t)n, -1);
  int count = 0;
  for (int v = 0; v < n; ++v)
    if (renum[(size_t)sub[(size_t)v]] < 0) renum[(size_t)sub[(size_t)v]] = count++;
  for (int v = 0; v < n; ++v) sub[(size_t)v] = renum[(size_t)sub[(size_t)v]];
  return count;
}

// One aggregation step: every adjacency entry (u, v) with u <= v contributes
// its weight to the community pair (c(u), c(v)).
Graph collapse(const Graph &g, const std::vector<int> &memb, int n_comm) {
  std::vector<WEdge> es;
  for (int u = 0; u < g.n; ++u) {
    for (int e = g.row[(size_t)u]; e < g.row[(size_t)u + 1]; ++e) {
      const int v = g.adj[(size_t)e];
      if (u > v) continue;
      int cu = memb[(size_t)u], cv = memb[(size_t)v];
      if (cu > cv) std::swap(cu, cv);
      es.emplace_back(std::make_pair(cu, cv), g.awt[(size_t)e]);
    }
  }
  return graph_from_edges(n_comm, es);
}

}  // namespace

std::vector<uint32_t> leiden(const std::vector<std::pair<int, int>> &edges, int n,
                             float resolution, uint64_t seed, int iterations) {
  std::vector<uint32_t> result;
  if (n <= 0) return result;
  result.assign((size_t)n, 0);
  const double gamma = (double)resolution;
  std::vector<WEdge> es;
  es.reserve(edges.size());
  for (const auto &e : edges) {
    const int u = e.first, v = e.second;
    if (u < 0 || v < 0 || u >= n || v >= n || u == v) continue;
    es.emplace_back(std::make_pair(std::min(u, v), std::max(u, v)), 1.0);
  }
  Graph g = graph_from_edges(n, es);
  if (iterations < 1) iterations = 1;
  std::vector<int> cur((size_t)n);
  std::iota(cur.begin(), cur.end(), 0);
  for (int it = 0; it < iterations; ++it) {
    for (int level = 0; level < 32; ++level) {
      std::vector<int> memb((size_t)g.n);
      std::iota(memb.begin(), memb.end(), 0);
      std::vector<double> tot = g.deg;
      if (local_moving(g, memb, tot, gamma) == 0) break;
      std::vector<int> sub;
      const int n_sub = refine(g, memb, sub, gamma,
                               seed + (uint64_t)it * 0x85ebca6bu +
                                   (uint64_t)level * 0x9e3779b1u);
      Graph g2 = collapse(g, sub, n_sub);
      for (int i = 0; i < n; ++i) cur[(size_t)i] = sub[(size_t)cur[(size_t)i]];
      g = std::move(g2);
      if (g.n <= 1) break;
    }
    if (g.n <= 1) break;
  }
  std::vector<int> renum((size_t)n, -1);
  int k = 0;
  for (int i = 0; i < n; ++i)
    if (renum[(size_t)cur[(size_t)i]] < 0) renum[(size_t)cur[(size_t)i]] = k++;
  for (int i = 0; i < n; ++i) result[(size_t)i] = (uint32_t)renum[(size_t)cur[(size_t)i]];
  return result;
}

}  // namespace ngia

extern "C" float ngia_leiden_resolution(uint32_t identity) {
  // (100 - |id - 50| * 2) / 100, clamped to [0, 1] (src/main.cu:114-116)
  float r = (100.0f - std::fabs((float)identity - 50.0f) * 2.0f) / 100.0f;
  if (r < 0.0f) r = 0.0f;
  return std::min(r, 1.0f);
}

extern "C" int ngia_leiden(const ngia_edge *h_edges, uint64_t m, uint32_t n, float resolution,
                           uint32_t seed, int iterations, uint32_t *h_cluster) {
  if (!h_cluster || (m && !h_edges) || n == 0 || n > 0x7FFFFFFEu) return NGIA_ERR_ARG;
  std::vector<std::pair<int, int>> e;
  e.reserve(m);
  for (uint64_t k = 0; k < m; ++k) e.emplace_back(h_edges[k].rep, h_edges[k].tar);
  std::vector<uint32_t> r = ngia::leiden(e, (int)n, resolution, seed, iterations);
  std::copy(r.begin(), r.end(), h_cluster);
  return NGIA_OK;
}
