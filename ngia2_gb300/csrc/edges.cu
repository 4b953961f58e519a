// edges.cu -- sort + unique of an edge list on the device
// (src/buildGraph.hpp:357-358: __gnu_parallel::sort then std::unique over
// tuple<int,int,float>).  Lexicographic (rep, tar, weight) order is built
// from three stable radix sorts, least significant field first; weights are
// non-negative floats, so their bit patterns sort like their values.
#include "kernels.cuh"

namespace ngia {

__global__ void edge_field_kernel(const ngia_edge *__restrict__ e,
                                  const uint32_t *__restrict__ perm, uint32_t m, int field,
                                  uint32_t *__restrict__ keys) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const ngia_edge x = e[perm ? perm[k] : k];
  keys[k] = field == 0 ? (uint32_t)x.rep
                       : (field == 1 ? (uint32_t)x.tar : __float_as_uint(x.weight));
}

__global__ void edge_gather_kernel(const ngia_edge *__restrict__ e,
                                   const uint32_t *__restrict__ perm, uint32_t m,
                                   ngia_edge *__restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m) out[k] = e[perm[k]];
}

__global__ void edge_new_flags_kernel(const ngia_edge *__restrict__ e, uint32_t m,
                                      uint32_t *__restrict__ flags) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  bool fresh = k == 0;
  if (!fresh) {
    const ngia_edge a = e[k - 1], b = e[k];
    fresh = a.rep != b.rep || a.tar != b.tar ||
            __float_as_uint(a.weight) != __float_as_uint(b.weight);
  }
  flags[k] = fresh ? 1u : 0u;
}

__global__ void edge_compact_kernel(const ngia_edge *__restrict__ e,
                                    const uint32_t *__restrict__ flags,
                                    const uint64_t *__restrict__ off, uint32_t m,
                                    ngia_edge *__restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m && flags[k]) out[off[k]] = e[k];
}

static int sort_unique(ngia_edge *d_edges, uint32_t *h_n, uint32_t n_nodes, char *w,
                       cudaStream_t s) {
  const uint32_t m = *h_n;
  auto take = [&](size_t bytes) {
    char *p = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(w) + 15) & ~uintptr_t(15));
    w = p + bytes;
    return p;
  };
  uint32_t *keys = reinterpret_cast<uint32_t *>(take((size_t)m * 4));
  uint32_t *skeys = reinterpret_cast<uint32_t *>(take((size_t)m * 4));
  uint32_t *pa = reinterpret_cast<uint32_t *>(take((size_t)m * 4));
  uint32_t *pb = reinterpret_cast<uint32_t *>(take((size_t)m * 4));
  ngia_edge *copy = reinterpret_cast<ngia_edge *>(take((size_t)m * sizeof(ngia_edge)));
  uint32_t *flags = reinterpret_cast<uint32_t *>(take((size_t)m * 4));
  uint64_t *off = reinterpret_cast<uint64_t *>(take((size_t)m * 8));
  uint64_t *total = reinterpret_cast<uint64_t *>(take(8));
  uint64_t *scan_tmp = reinterpret_cast<uint64_t *>(take(scan_scratch_bytes(m)));
  void *sort_tmp = take(radix_sort_scratch_bytes(m, 1));
  const uint32_t blocks = ceil_div(m, 256u);
  const int node_bits = bits_for(n_nodes ? n_nodes - 1 : 0);
  // weight, then tar, then rep (stable): final order is (rep, tar, weight)
  edge_field_kernel<<<blocks, 256, 0, s>>>(d_edges, nullptr, m, 2, keys);
  NGIA_LAUNCHED();
  NGIA_TRY(radix_sort_pairs(keys, nullptr, skeys, pa, m, 1, 0, 32, sort_tmp, s));
  edge_field_kernel<<<blocks, 256, 0, s>>>(d_edges, pa, m, 1, keys);
  NGIA_LAUNCHED();
  NGIA_TRY(radix_sort_pairs(keys, pa, skeys, pb, m, 1, 0, node_bits > 0 ? node_bits : 8,
                            sort_tmp, s));
  edge_field_kernel<<<blocks, 256, 0, s>>>(d_edges, pb, m, 0, keys);
  NGIA_LAUNCHED();
  NGIA_TRY(radix_sort_pairs(keys, pb, skeys, pa, m, 1, 0, node_bits > 0 ? node_bits : 8,
                            sort_tmp, s));
  edge_gather_kernel<<<blocks, 256, 0, s>>>(d_edges, pa, m, copy);
  NGIA_LAUNCHED();
  edge_new_flags_kernel<<<blocks, 256, 0, s>>>(copy, m, flags);
  NGIA_LAUNCHED();
  NGIA_TRY(exclusive_scan_u64(flags, off, m, total, scan_tmp, s));
  edge_compact_kernel<<<blocks, 256, 0, s>>>(copy, flags, off, m, d_edges);
  NGIA_LAUNCHED();
  uint64_t h_total = 0;
  NGIA_CUDA(cudaMemcpyAsync(&h_total, total, 8, cudaMemcpyDeviceToHost, s));
  NGIA_CUDA(cudaStreamSynchronize(s));
  *h_n = (uint32_t)h_total;
  return NGIA_OK;
}

}  // namespace ngia

extern "C" int ngia_sort_unique_edges(ngia_edge *d_edges, uint32_t *h_n, uint32_t n_nodes,
                                      void *stream) {
  using namespace ngia;
  if (!h_n) return NGIA_ERR_ARG;
  const uint32_t m = *h_n;
  if (m == 0) return NGIA_OK;
  if (!d_edges) return NGIA_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  const size_t bytes = (size_t)m * (4 * 5 + sizeof(ngia_edge) + 8) + scan_scratch_bytes(m) +
                       radix_sort_scratch_bytes(m, 1) + 16 * 16;
  void *scratch = nullptr;
  cudaError_t e = cudaMallocAsync(&scratch, bytes, s);
  if (e != cudaSuccess) {
    cuda_fail(e);
    return NGIA_ERR_NOMEM;
  }
  int st = sort_unique(d_edges, h_n, n_nodes, static_cast<char *>(scratch), s);
  e = cudaFreeAsync(scratch, s);
  if (st == NGIA_OK && e != cudaSuccess) st = cuda_fail(e);
  if (st == NGIA_OK) {
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_fail(e);
  }
  return st;
}
