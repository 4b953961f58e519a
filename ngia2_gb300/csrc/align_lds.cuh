// align_lds.cuh -- the batched aligner's main kernel body: banded bit-parallel
// LCS with match masks read from per-thread tables in shared memory
// (internal header).
//
// Same recurrence and window as lcs_window (align.cuh); what changes is where
// the match mask comes from.  When a row block enters the band its 15 match
// masks (one per nonzero residue code: bit r set when row r has that code)
// are written once into the thread's table; every column step then reads the
// mask of each live row word with one shared-memory load, so the integer ALU
// only does the three operations of the LCS update per word
//     t = V & M;   s = V + t + carry;   V = s | (V ^ t)
// and the column code and table address are formed by integer multiply-adds
// (the FMA pipe).  Targets are read as 4-bit codes packed eight per word
// (nibble layout, first residue in the high nibble).
//
// Registers.  Window word of row r lives in V[r % W], so nothing moves when
// the band slides: a retiring row is counted and reset to all-ones, its table
// slot is cleared (zero masks keep an unvisited word all-ones), and an
// entering row only has its table written.  The rotation J0 % W is a template
// parameter of the column-block body, one instance per rotation.
//
// Shared memory per warp: [16 codes][W slots][32 lanes] words, so the 32
// lanes of a load hit 32 different banks.
#pragma once

#include <utility>

#include "align.cuh"

#ifndef NGIA_LDS_UNROLL
#define NGIA_LDS_UNROLL 2  // column steps unrolled per loop trip
#endif
#ifndef NGIA_LDS_PREFETCH
#define NGIA_LDS_PREFETCH 1  // 1: load the next block's words one block ahead
#endif

namespace ngia {

constexpr int kLdsUnroll = NGIA_LDS_UNROLL;

// K = entries per row block: 16 (all residue codes), or 8 / 5 when the
// database uses at most 7 / 4 nonzero codes and the records were recoded
// densely (the table, and so the shared memory per thread, shrinks to a half /
// under a third; nucleotides take 5).
template <int W, int K = 16>
struct LdsTable {
  uint32_t *base;  // this thread's column of the warp's table
  uint64_t inv;    // nibble d = residue code that aligner code d stands for
                   // (K = 8: the rows come as code planes, see fill)
  __device__ __forceinline__ uint32_t *slot(uint32_t s) const { return base + s * 32; }
  static constexpr uint32_t kCodeStride = W * 32;  // words between codes
  __device__ __forceinline__ void clear(uint32_t s) const {
    uint32_t *p = slot(s);
#pragma unroll
    for (int c = 1; c < K; ++c) p[c * kCodeStride] = 0u;
  }
  // masks of one row block from its four bit planes
  __device__ __forceinline__ void fill(uint32_t s, const uint4 &pl) const {
    uint32_t *p = slot(s);
    if constexpr (K == 16) {
      const uint32_t lo[4] = {~pl.x & ~pl.y, pl.x & ~pl.y, ~pl.x & pl.y, pl.x & pl.y};
      const uint32_t hi[4] = {~pl.z & ~pl.w, pl.z & ~pl.w, ~pl.z & pl.w, pl.z & pl.w};
#pragma unroll
      for (int c = 1; c < 16; ++c) p[c * kCodeStride] = lo[c & 3] & hi[c >> 2];
    } else {  // K = 5 or 8: the code planes (aligner code bits in planes 0-2)
#pragma unroll
      for (int d = 1; d < K; ++d)
        p[d * kCodeStride] = ((d & 1) ? pl.x : ~pl.x) & ((d & 2) ? pl.y : ~pl.y) &
                             ((d & 4) ? pl.z : ~pl.z);
    }
  }
};

__device__ __forceinline__ uint4 load4(const uint32_t *p) {
  return make_uint4(__ldg(p), __ldg(p + 1), __ldg(p + 2), __ldg(p + 3));
}

// One column step over the window in row order (word m of the run = slot
// (R + m) % W), the masks M already in row order.
template <int W, int R, int... I>
__device__ __forceinline__ void column_run(uint32_t (&V)[W], const uint32_t (&M)[W],
                                           std::integer_sequence<int, I...>) {
  lcs_run<W>(V[(R + I) % W]..., M[I]...);
}

// 32 column steps of one column block with the window rotated by R.
template <int W, int R>
__device__ __forceinline__ void lds_columns(uint32_t (&V)[W], const uint32_t *tab,
                                            const uint4 &nib) {
  uint32_t w0 = nib.x, w1 = nib.y, w2 = nib.z, w3 = nib.w;
#pragma unroll 1
  for (int q = 0; q < 4; ++q) {
    uint32_t x = w0;  // the code words move down one per 8 columns
    w0 = w1;
    w1 = w2;
    w2 = w3;
#pragma unroll kLdsUnroll
    for (int k = 0; k < 8; ++k) {
      uint32_t code;
      asm("mul.hi.u32 %0, %1, 16;" : "=r"(code) : "r"(x));
      asm("mul.lo.u32 %0, %0, 16;" : "+r"(x));
      const uint32_t *row = tab + code * LdsTable<W>::kCodeStride;
      uint32_t M[W];
#pragma unroll
      for (int m = 0; m < W; ++m) M[m] = row[((R + m) % W) * 32];
      column_run<W, R>(V, M, std::make_integer_sequence<int, W>{});
    }
  }
}

// Rows entering the band at this column block, with the planes of the one
// row that was prefetched during the previous block.
struct Entering {
  uint32_t act;     // rows loaded so far
  uint32_t j1;      // rows to have loaded after this block
  uint32_t pf_row;  // row whose planes are in pf
  uint4 pf;
};

// One column block at rotation R: retire the row leaving the band, load the
// rows entering it, then the 32 column steps.
template <int W, int R, typename Tab>
__device__ __forceinline__ void lds_block(uint32_t (&V)[W], const Tab &tab,
                                          const uint32_t *__restrict__ rep, const uint4 &nib,
                                          bool retire, Entering &in, uint32_t &lcs) {
  if (retire) {
    constexpr int out = (R + W - 1) % W;
    lcs += __popc(~V[out]);
    V[out] = kFull;
    tab.clear(out);
  }
  for (; in.act < in.j1; ++in.act)
    tab.fill(in.act % W, in.act == in.pf_row ? in.pf : load4(rep + 1 + 4 * in.act));
  lds_columns<W, R>(V, tab.base, nib);
}

template <int W, typename Tab, int R = 0>
__device__ __forceinline__ void lds_dispatch(uint32_t rot, uint32_t (&V)[W], const Tab &tab,
                                             const uint32_t *__restrict__ rep,
                                             const uint4 &nib, bool retire, Entering &in,
                                             uint32_t &lcs) {
  if constexpr (R < W) {
    if (rot == R) {
      lds_block<W, R>(V, tab, rep, nib, retire, in, lcs);
      return;
    }
    lds_dispatch<W, Tab, R + 1>(rot, V, tab, rep, nib, retire, in, lcs);
  }
}

// LCS of the banded computation; requires b.width <= W.  tar_nib points at
// the target's nibble words (position 8k..8k+7 in word k).  The next column
// block's code words and the next entering row's planes are loaded one block
// ahead so that their latency hides behind the current block's steps.
template <int W, typename Tab>
__device__ inline uint32_t lcs_lds(const uint32_t *__restrict__ rep,
                                   const uint32_t *__restrict__ tar_nib, const Band &b,
                                   const Tab &tab, uint32_t &blocks) {
#pragma unroll 1
  for (uint32_t s = 0; s < (uint32_t)W; ++s) {
    tab.clear(s);
    tab.slot(s)[0] = 0u;
  }
  uint32_t V[W];
#pragma unroll
  for (int m = 0; m < W; ++m) V[m] = kFull;
  uint32_t lcs = 0;
  Entering in{0u, 0u, kFull, make_uint4(0u, 0u, 0u, 0u)};
  uint4 cur = b.nc ? load4(tar_nib) : make_uint4(0u, 0u, 0u, 0u);
  for (uint32_t i = 0; i < b.nc; ++i) {
    const uint32_t j0 = i > b.ls ? i - b.ls : 0;
    in.j1 = (i + b.rs < b.nr) ? i + b.rs : b.nr;
    const uint32_t j1n = (i + 1 + b.rs < b.nr) ? i + 1 + b.rs : b.nr;
    const bool more = NGIA_LDS_PREFETCH && i + 1 < b.nc;
    const uint4 nxt = more ? load4(tar_nib + 4 * (i + 1)) : cur;
    uint4 pf_next = in.pf;
    uint32_t pf_row_next = in.pf_row;
    if (more && j1n > in.j1) {
      pf_row_next = j1n - 1;
      pf_next = load4(rep + 1 + 4 * pf_row_next);
    }
    if (!NGIA_LDS_PREFETCH) cur = load4(tar_nib + 4 * i);
    lds_dispatch<W>(j0 % W, V, tab, rep, cur, i > b.ls, in, lcs);
    cur = nxt;
    in.pf = pf_next;
    in.pf_row = pf_row_next;
    uint32_t z = lcs;
#pragma unroll
    for (int m = 0; m < W; ++m) z += __popc(~V[m]);
    if (!may_reach_threshold(z, 32 * (i + 1), b)) {  // score 0 already certain
      blocks = i + 1;
      return 0;
    }
  }
#pragma unroll
  for (int m = 0; m < W; ++m) lcs += __popc(~V[m]);
  blocks = b.nc;
  return lcs;
}

// Threads per block of the shared-memory aligner for width W (64*W bytes of
// table per thread).
#ifndef NGIA_LDS_THREADS
#define NGIA_LDS_THREADS 64
#endif
__host__ __device__ constexpr int lds_threads(int W) { return W > 0 ? NGIA_LDS_THREADS : 0; }
__host__ __device__ constexpr size_t lds_smem_bytes(int W, int K) {
  return (size_t)lds_threads(W) * K * W * 4;
}

}  // namespace ngia
