// align_stream.cuh -- persistent shared-memory aligner: each lane of a warp
// aligns its own stream of pairs (internal header).
//
// Same recurrence, tables and column steps as align_lds.cuh.  What changes is
// how the 32 lanes of a warp share the instruction stream.  With one pair per
// lane for the whole launch, lanes whose pairs are shorter, or whose score is
// settled early, idle until the warp's slowest pair ends, and lanes whose
// bands start at different row offsets rotate their windows differently, so
// the rotation switch diverges.  Here:
//
// Virtual rows.  A pair's window holds rows j0v .. j0v + W - 1 with
// j0v = i - ls at column block i; rows below 0 are virtual (all ones, zero
// masks): they pass a zero carry up unchanged, which is exactly the band's
// zero carry into its lowest live row J0 = max(i - ls, 0).  Row r lives in
// slot (base + r) % W with base = (g0 + ls) % W, g0 being the warp step at
// which the pair's first column block runs.  At warp step g the window's
// lowest row then sits in slot g % W in every lane: the rotation is uniform
// across the warp whatever each lane's pair is.  The window covers every live
// row [J0, J1) when ls + min(rs, nr) <= W, the width these classes are
// binned by.
//
// Streams.  A lane whose pair ends (last column block, or a score of 0
// already certain) writes the score, resets its window and takes the next
// pair of its warp's chunk (32 pairs claimed from the class's queue with one
// atomic), so the lanes stay busy until the queue drains.  Pairs are queued
// longest first.
#pragma once

#include "align_lds.cuh"

namespace ngia {

// Threads per block of the streaming kernels (each warp owns its tables).
constexpr int kStreamThreads = 64;
// Resident blocks per SM the register allocation must allow (1: no bound).
#ifndef NGIA_STREAM_MIN_BLOCKS
#define NGIA_STREAM_MIN_BLOCKS 1
#endif

__host__ __device__ constexpr size_t stream_smem_bytes(int W, int K) {
  return (size_t)kStreamThreads * K * W * 4;
}

// A queued pair, as staged for a refill.
struct PairDesc {
  uint32_t p, lr, lt;
  uint64_t ro, to;  // record offsets of rep and target
};

__device__ __forceinline__ uint64_t shfl64(uint64_t v, uint32_t src) {
  const uint32_t lo = __shfl_sync(kFull, (uint32_t)v, src);
  const uint32_t hi = __shfl_sync(kFull, (uint32_t)(v >> 32), src);
  return ((uint64_t)hi << 32) | lo;
}

// One lane's pair.
struct StreamPair {
  const uint32_t *rep;  // rep record (length word, then bit planes)
  const uint32_t *tar;  // target's nibble code words
  uint32_t p;           // pair index (score slot)
  uint32_t i;           // current column block
  uint32_t nc, nr, rs, ls;
  uint32_t act;         // rows entered so far
  uint32_t in_slot;     // slot of row `act`
  uint32_t lcs;         // zeros of the retired rows
  uint32_t lr, lt;
  uint4 cur;            // code words of block i
  uint4 pf;             // planes of row pf_row, loaded one block ahead
  uint32_t pf_row;
  bool active;
};

// What the early exit needs to know about a pair after a block.
struct BlockEnd {
  int32_t left;  // target columns after this block
  int32_t lr;    // rep length
  int32_t row0;  // first row of window word 0 (32 (i - ls); negative: virtual)
};

// Retire the window word leaving at rotation R (its zeros are returned), then
// the block's 32 column steps, then, in row order (static at rotation R):
//   total = the LCS so far (zeros of the retired rows and of the window),
//   ub    = an upper bound of the pair's final LCS.
// The banded LCS is the best monotone path through the matrix counting
// matches in band cells only (rows below the band hold their values, rows
// above it enter all ones with empty masks).  Such a path crosses the last
// column done at some row j, so the final LCS is at most
//   L(j) + min(columns left, Lr - j)
// with L(j) the zeros of rows 0..j now.  Taken at word granularity (the
// zeros through the end of a word, the rows above its start) and over the
// retired rows (at most all retired zeros + columns left), the maximum is an
// upper bound no larger than total + columns left.
template <int W, int R = 0>
__device__ __forceinline__ uint32_t columns_dispatch(uint32_t rot, uint32_t (&V)[W],
                                                     const uint32_t *tab, const uint4 &nib,
                                                     uint32_t retired, const BlockEnd &be,
                                                     uint32_t &total, uint32_t &ub) {
  if constexpr (R < W) {
    if (rot == R) {
      constexpr int out = (R + W - 1) % W;
      const uint32_t z = __popc(~V[out]);
      V[out] = kFull;
      lds_columns<W, R>(V, tab, nib);
      int32_t p = (int32_t)(retired + z);
      int32_t best = p + min(be.left, be.lr);
#pragma unroll
      for (int m = 0; m < W; ++m) {
        p += __popc(~V[(R + m) % W]);
        const int32_t above = max(be.lr - (be.row0 + 32 * m), 0);
        best = max(best, p + min(be.left, above));
      }
      total = (uint32_t)p;
      ub = (uint32_t)best;
      return z;
    }
    return columns_dispatch<W, R + 1>(rot, V, tab, nib, retired, be, total, ub);
  }
  return 0;
}

// One column block at warp rotation `rot`: retire the row leaving the window,
// enter the rows reaching the band, 32 column steps.  Only the retire and the
// column steps are instantiated per rotation (W copies of a short loop); the
// table work indexes its slots at run time, so the code of a wide class stays
// small enough for the instruction cache.
template <int W, typename Tab>
__device__ __forceinline__ void stream_block(uint32_t rot, uint32_t (&V)[W], const Tab &tab,
                                             StreamPair &sp, uint32_t &total, uint32_t &ub) {
  const uint32_t out = rot == 0 ? (uint32_t)W - 1 : rot - 1;  // (rot + W - 1) % W
  // the next block's code words and entering row (J1 moves up at most one row
  // per block), loaded now so that their latency hides behind this block
  const bool more = sp.i + 1 < sp.nc;
  const uint4 nxt = more ? load4(sp.tar + 4 * (sp.i + 1)) : sp.cur;
  const uint32_t j1 = sp.i + sp.rs < sp.nr ? sp.i + sp.rs : sp.nr;
  const uint32_t j1n = sp.i + 1 + sp.rs < sp.nr ? sp.i + 1 + sp.rs : sp.nr;
  uint4 pfn = sp.pf;
  uint32_t pfn_row = sp.pf_row;
  if (more && j1n > j1) {
    pfn_row = j1n - 1;
    pfn = load4(sp.rep + 1 + 4 * pfn_row);
  }
  tab.clear(out);
  for (; sp.act < j1; ++sp.act) {
    tab.fill(sp.in_slot, sp.act == sp.pf_row ? sp.pf : load4(sp.rep + 1 + 4 * sp.act));
    sp.in_slot = sp.in_slot + 1 == (uint32_t)W ? 0u : sp.in_slot + 1;
  }
  const int32_t cols = 32 * (int32_t)(sp.i + 1);
  const BlockEnd be{(int32_t)sp.lt > cols ? (int32_t)sp.lt - cols : 0, (int32_t)sp.lr,
                    32 * ((int32_t)sp.i - (int32_t)sp.ls)};
  sp.lcs += columns_dispatch<W>(rot, V, tab.base, sp.cur, sp.lcs, be, total, ub);
  sp.cur = nxt;
  sp.pf = pfn;
  sp.pf_row = pfn_row;
}

// The persistent kernel body of one width class.  `order[begin, end)` lists
// the class's pairs; `cursor` counts the pairs taken (zero at launch).
// Returns the column blocks x W computed by this lane.
template <int W, int K>
__device__ inline uint32_t align_stream(const uint32_t *__restrict__ packed,
                                        const uint32_t *__restrict__ nib, uint64_t inv,
                                        const uint64_t *__restrict__ offs,
                                        const uint2 *__restrict__ pairs,
                                        const uint32_t *__restrict__ order, uint32_t begin,
                                        uint32_t end, unsigned int *__restrict__ cursor,
                                        uint32_t *__restrict__ scores, float t,
                                        int fma_mode, uint32_t *smem) {
  const uint32_t lane = threadIdx.x & 31u;
  const LdsTable<W, K> tab{smem + (threadIdx.x >> 5) * (K * W * 32) + lane, inv};
#pragma unroll 1
  for (uint32_t s = 0; s < (uint32_t)W; ++s) {
    tab.clear(s);
    tab.slot(s)[0] = 0u;  // code 0 matches nothing
  }
  uint32_t V[W];
#pragma unroll
  for (int m = 0; m < W; ++m) V[m] = kFull;
  StreamPair sp;
  sp.active = false;
  // Pair descriptors, staged per warp: lane l of A holds the l-th pair of the
  // warp's current chunk of 32 (claimed with one atomic and loaded together:
  // queue slot -> pair -> record offsets -> lengths), so a refill waits on
  // global memory once per 32 pairs instead of once per pair.
  PairDesc A{};
  uint32_t a_count = 0, a_used = 0;      // warp-uniform
  bool queue_empty = false;
  uint32_t done = 0, g = 0;
  for (;;) {
    // lanes without a pair take the next descriptors of A, a new chunk
    // being claimed when A runs out
    uint32_t need = __ballot_sync(kFull, !sp.active);
    while (need) {
      if (a_used == a_count) {
        if (queue_empty) break;
        uint32_t first = 0;
        if (lane == 0) first = atomicAdd(cursor, 32u);
        first = __shfl_sync(kFull, first, 0);
        const uint32_t size = end - begin;
        a_count = first < size ? min(size - first, 32u) : 0u;
        a_used = 0;
        if (a_count == 0) {
          queue_empty = true;
          break;
        }
        if (lane < a_count) {
          A.p = order[begin + first + lane];
          const uint2 pr = pairs[A.p];
          A.ro = offs[pr.x];
          A.to = offs[pr.y];
          A.lr = __ldg(packed + A.ro);
          A.lt = __ldg(packed + A.to);
        }
      }
      const uint32_t rank = __popc(need & ((1u << lane) - 1u));
      const uint32_t take = min((uint32_t)__popc(need), a_count - a_used);
      const uint32_t src = a_used + (rank < take ? rank : 0u);
      const uint32_t p = __shfl_sync(kFull, A.p, src);
      const uint32_t lr = __shfl_sync(kFull, A.lr, src);
      const uint32_t lt = __shfl_sync(kFull, A.lt, src);
      const uint64_t ro = shfl64(A.ro, src), to = shfl64(A.to, src);
      const bool mine = (need >> lane & 1u) && rank < take;
      if (mine) {
        const Band b = make_band(lr, lt, t, fma_mode);
        if (b.nc == 0) {
          scores[p] = identity_score(0u, lr, lt, t);
        } else {
          sp.rep = packed + ro;
          sp.tar = nib + to + 1;
          sp.lr = lr;
          sp.lt = lt;
          sp.p = p;
          sp.i = 0;
          sp.nc = b.nc;
          sp.nr = b.nr;
          sp.rs = b.rs;
          sp.ls = b.ls;
          sp.act = 0;
          sp.in_slot = (g + b.ls) % (uint32_t)W;
          sp.lcs = 0;
          sp.cur = load4(sp.tar);
          sp.pf_row = kFull;
          sp.active = true;
        }
      }
      a_used += take;
      need &= ~__ballot_sync(kFull, mine);
      // lanes whose pair needed no alignment ask again
      need |= __ballot_sync(kFull, mine && !sp.active);
    }
    if (!__any_sync(kFull, sp.active)) {
      if (queue_empty) break;
      continue;
    }
    uint32_t total = 0, ub = 0;
    if (sp.active) stream_block<W>(g % (uint32_t)W, V, tab, sp, total, ub);
    ++g;
    if (sp.active) {
      ++sp.i;
      done += W;
      const bool last = sp.i >= sp.nc;
      if (last || !lcs_may_reach(ub, sp.lr, sp.lt, t)) {
        scores[sp.p] = last ? identity_score(total, sp.lr, sp.lt, t) : 0u;
        sp.active = false;
#pragma unroll
        for (int m = 0; m < W; ++m) V[m] = kFull;
#pragma unroll 1
        for (uint32_t s = 0; s < (uint32_t)W; ++s) tab.clear(s);
      }
    }
  }
  return done;
}

}  // namespace ngia
