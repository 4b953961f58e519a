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

#include "align.cuh"

namespace ngia {

template <int W>
struct LdsTable {
  uint32_t *base;  // this thread's column of the warp's table
  __device__ __forceinline__ uint32_t *slot(uint32_t s) const { return base + s * 32; }
  static constexpr uint32_t kCodeStride = W * 32;  // words between codes
  __device__ __forceinline__ void clear(uint32_t s) const {
    uint32_t *p = slot(s);
#pragma unroll
    for (int c = 1; c < 16; ++c) p[c * kCodeStride] = 0u;
  }
  // masks of one row block from its four bit planes
  __device__ __forceinline__ void fill(uint32_t s, const uint32_t *rb) const {
    const uint32_t p0 = __ldg(rb), p1 = __ldg(rb + 1), p2 = __ldg(rb + 2), p3 = __ldg(rb + 3);
    const uint32_t lo[4] = {~p0 & ~p1, p0 & ~p1, ~p0 & p1, p0 & p1};
    const uint32_t hi[4] = {~p2 & ~p3, p2 & ~p3, ~p2 & p3, p2 & p3};
    uint32_t *p = slot(s);
#pragma unroll
    for (int c = 1; c < 16; ++c) p[c * kCodeStride] = lo[c & 3] & hi[c >> 2];
  }
};

// 32 column steps of one column block with the window rotated by R.
template <int W, int R>
__device__ __forceinline__ void lds_columns(uint32_t (&V)[W], const uint32_t *tab,
                                            const uint32_t *__restrict__ nib) {
#pragma unroll 1
  for (int q = 0; q < 4; ++q) {
    uint32_t x = __ldg(nib + q);
#pragma unroll 4
    for (int k = 0; k < 8; ++k) {
      uint32_t code;
      asm("mul.hi.u32 %0, %1, 16;" : "=r"(code) : "r"(x));
      asm("mul.lo.u32 %0, %0, 16;" : "+r"(x));
      const uint32_t *row = tab + code * LdsTable<W>::kCodeStride;
      uint32_t a[W], t[W], s[W];
#pragma unroll
      for (int m = 0; m < W; ++m) {
        const int slot = (R + m) % W;
        a[m] = V[slot];
        t[m] = a[m] & row[slot * 32];
      }
      add_words<W, false>(s, a, t, 0);
#pragma unroll
      for (int m = 0; m < W; ++m) V[(R + m) % W] = s[m] | (a[m] ^ t[m]);
    }
  }
}

// One column block at rotation R: retire the row leaving the band, load the
// rows entering it, then the 32 column steps.
template <int W, int R>
__device__ __forceinline__ void lds_block(uint32_t (&V)[W], const LdsTable<W> &tab,
                                          const uint32_t *__restrict__ rep,
                                          const uint32_t *__restrict__ nib, bool retire,
                                          uint32_t &act, uint32_t j1, uint32_t &lcs) {
  if (retire) {
    constexpr int out = (R + W - 1) % W;
    lcs += __popc(~V[out]);
    V[out] = kFull;
    tab.clear(out);
  }
  for (; act < j1; ++act) tab.fill(act % W, rep + 1 + 4 * act);
  lds_columns<W, R>(V, tab.base, nib);
}

template <int W, int R = 0>
__device__ __forceinline__ void lds_dispatch(uint32_t rot, uint32_t (&V)[W],
                                             const LdsTable<W> &tab,
                                             const uint32_t *__restrict__ rep,
                                             const uint32_t *__restrict__ nib, bool retire,
                                             uint32_t &act, uint32_t j1, uint32_t &lcs) {
  if constexpr (R < W) {
    if (rot == R) {
      lds_block<W, R>(V, tab, rep, nib, retire, act, j1, lcs);
      return;
    }
    lds_dispatch<W, R + 1>(rot, V, tab, rep, nib, retire, act, j1, lcs);
  }
}

// LCS of the banded computation; requires b.width <= W.  tar_nib points at
// the target's nibble words (position 8k..8k+7 in word k).
template <int W>
__device__ inline uint32_t lcs_lds(const uint32_t *__restrict__ rep,
                                   const uint32_t *__restrict__ tar_nib, const Band &b,
                                   const LdsTable<W> &tab) {
#pragma unroll 1
  for (uint32_t s = 0; s < (uint32_t)W; ++s) {
    tab.clear(s);
    tab.slot(s)[0] = 0u;
  }
  uint32_t V[W];
#pragma unroll
  for (int m = 0; m < W; ++m) V[m] = kFull;
  uint32_t lcs = 0, act = 0;
  for (uint32_t i = 0; i < b.nc; ++i) {
    const uint32_t j0 = i > b.ls ? i - b.ls : 0;
    const uint32_t j1 = (i + b.rs < b.nr) ? i + b.rs : b.nr;
    lds_dispatch<W>(j0 % W, V, tab, rep, tar_nib + 4 * i, i > b.ls, act, j1, lcs);
  }
#pragma unroll
  for (int m = 0; m < W; ++m) lcs += __popc(~V[m]);
  return lcs;
}

// Threads per block of the shared-memory aligner for width W (64*W bytes of
// table per thread).
#ifndef NGIA_LDS_THREADS
#define NGIA_LDS_THREADS 64
#endif
__host__ __device__ constexpr int lds_threads(int W) { return W > 0 ? NGIA_LDS_THREADS : 0; }
__host__ __device__ constexpr size_t lds_smem_bytes(int W) {
  return (size_t)lds_threads(W) * 16 * W * 4;
}

}  // namespace ngia
