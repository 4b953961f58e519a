// align.cuh -- banded bit-parallel LCS of one (rep, tar) pair (internal header).
//
// Restates BuildGraph::kernel_dynamic (src/buildGraph.hpp:192-253), identical
// to FastClustering::kernel_dynamic (src/fastClustering.hpp:183-244).
//
// Recurrence.  Rows are the representative's residues, columns the target's.
// A row bit is 1 while the row is unmatched.  One column step with match mask
// M (rows whose 4-bit code equals the column's code; code 0 matches nothing)
// is the bit-parallel LCS update
//     V' = (V + (V & M) + carry_in) | (V & ~M)
// applied to the multi-word vector of the rows inside the band, the carry
// rippling upward from the band's lowest row block (carry 0 there).  The
// reference applies it block by block (32 columns x 32 rows, column carries
// kept in a shift register); here one column step updates every live row
// word at once, which is the same set of dependencies evaluated in another
// order, and the word-to-word carry is the hardware carry flag.
//
// Window form (lcs_window<W>).  Live row blocks [J0(I), J1(I)) never exceed
// min(ls + rs, nr) words and both ends advance by at most one block per
// column block, so the live rows sit in a register window V[0..W) based at
// J0: when J0 advances, V[0] retires into the LCS sum and the window shifts
// down; a row block entering at J1 gets its four bit planes loaded.  Window
// slots above J1 hold all-ones with zero planes: zero planes mean code 0,
// which matches nothing, so those words stay all-ones and only pass the carry
// through -- exactly the "not yet visited" state of the reference.
//
// Match masks are computed from the bit planes with no lookup table:
//   u = (P0 & T0) | (~P0 & B);  u &= ~(Pe ^ Te) for e = 1..3;  t = V & u
// where Te = all-ones if bit e of the column code is set, B = ~T0 & (T1|T2|T3)
// (so a zero column code gives u = 0).  Since t = V & M is a subset of V,
// V & ~M = V ^ t and the update is V' = (V + t + c) | (V ^ t).
#pragma once

#include "carry_chain.cuh"
#include "common.cuh"

namespace ngia {

// One chunk of C words of a multi-word add (carry in when CIN, carry out when
// COUT), dispatched to the PTX chains.
template <int C, bool CIN, bool COUT>
__device__ __forceinline__ void add_chunk(uint32_t *s, const uint32_t *a, const uint32_t *b,
                                          uint32_t cin, uint32_t &cout) {
#define NGIA_CHUNK(N)                                              \
  if constexpr (C == N) {                                          \
    if constexpr (CIN && COUT) add_chain##N##_cc(s, a, b, cin, cout); \
    else if constexpr (CIN) add_chain##N##_cn(s, a, b, cin);       \
    else if constexpr (COUT) add_chain##N##_zc(s, a, b, cout);     \
    else add_chain##N##_zn(s, a, b);                               \
  }
  NGIA_CHUNK(2)
  NGIA_CHUNK(4)
  NGIA_CHUNK(8)
#undef NGIA_CHUNK
}

// s[0..W) = a + b as one W-word number (carry in = cin != 0 when CIN; W even
// when CIN or W > 16).
template <int W, bool CIN>
__device__ __forceinline__ void add_words(uint32_t *s, const uint32_t *a,
                                          const uint32_t *b, uint32_t cin) {
  constexpr int C = W >= 8 ? 8 : (W >= 4 ? 4 : 2);
  uint32_t c = 0;
  if constexpr (!CIN && W <= 16) {
    add_run<W>(s, a, b);
  } else if constexpr (W == C) {
    static_assert(W % 2 == 0, "window width must be even");
    add_chunk<C, CIN, false>(s, a, b, cin, c);
  } else {
    add_chunk<C, CIN, true>(s, a, b, cin, c);
    add_words<W - C, true>(s + C, a + C, b + C, c);
  }
}

// Column-code masks of a target block, one column per step.  The four planes
// are bit-reversed once per block so that column k's bits sit in bit 31 after
// k left shifts; Te = arithmetic shift of that sign bit across the word.
struct ColMask {
  uint32_t T0, T1, T2, T3, B;
};
struct ColumnPlanes {
  uint32_t r0, r1, r2, r3;
  __device__ __forceinline__ explicit ColumnPlanes(const uint32_t *tb) {
#ifdef __CUDA_ARCH__
    r0 = __brev(__ldg(tb));
    r1 = __brev(__ldg(tb + 1));
    r2 = __brev(__ldg(tb + 2));
    r3 = __brev(__ldg(tb + 3));
#endif
  }
  // masks of the next column, then advance
  __device__ __forceinline__ ColMask next() {
    ColMask m;
    m.T0 = (uint32_t)((int32_t)r0 >> 31);
    m.T1 = (uint32_t)((int32_t)r1 >> 31);
    m.T2 = (uint32_t)((int32_t)r2 >> 31);
    m.T3 = (uint32_t)((int32_t)r3 >> 31);
    m.B = ~m.T0 & (m.T1 | m.T2 | m.T3);
    r0 <<= 1;
    r1 <<= 1;
    r2 <<= 1;
    r3 <<= 1;
    return m;
  }
};

__device__ __forceinline__ uint32_t match_and(uint32_t v, uint32_t p0, uint32_t p1,
                                              uint32_t p2, uint32_t p3,
                                              const ColMask &c) {
  uint32_t u = (p0 & c.T0) | (~p0 & c.B);
  u &= ~(p1 ^ c.T1);
  u &= ~(p2 ^ c.T2);
  u &= ~(p3 ^ c.T3);
  return v & u;
}

template <int W>
__device__ __forceinline__ void window_step(uint32_t (&V)[W], const uint32_t (&P0)[W],
                                            const uint32_t (&P1)[W],
                                            const uint32_t (&P2)[W],
                                            const uint32_t (&P3)[W],
                                            const ColMask &c) {
  uint32_t t[W], s[W];
#pragma unroll
  for (int m = 0; m < W; ++m) t[m] = match_and(V[m], P0[m], P1[m], P2[m], P3[m], c);
  add_words<W, false>(s, V, t, 0);
#pragma unroll
  for (int m = 0; m < W; ++m) V[m] = s[m] | (V[m] ^ t[m]);
}

// LCS of the banded computation, window form; requires b.width <= W.
template <int W>
// `blocks` receives the column blocks processed (fewer than b.nc after an
// early exit).
__device__ inline uint32_t lcs_window(const uint32_t *__restrict__ rep,
                                      const uint32_t *__restrict__ tar, const Band &b,
                                      uint32_t &blocks) {
  uint32_t V[W], P0[W], P1[W], P2[W], P3[W];
#pragma unroll
  for (int m = 0; m < W; ++m) {
    V[m] = kFull;
    P0[m] = P1[m] = P2[m] = P3[m] = 0;
  }
  uint32_t lcs = 0, act = 0;  // act = row blocks loaded so far
  for (uint32_t i = 0; i < b.nc; ++i) {
    if (i > b.ls) {  // J0 advances: retire the bottom row block
      lcs += __popc(~V[0]);
#pragma unroll
      for (int m = 0; m < W - 1; ++m) {
        V[m] = V[m + 1];
        P0[m] = P0[m + 1];
        P1[m] = P1[m + 1];
        P2[m] = P2[m + 1];
        P3[m] = P3[m + 1];
      }
      V[W - 1] = kFull;
      P0[W - 1] = P1[W - 1] = P2[W - 1] = P3[W - 1] = 0;
    }
    const uint32_t j0 = i > b.ls ? i - b.ls : 0;
    const uint32_t j1 = (i + b.rs < b.nr) ? i + b.rs : b.nr;
    for (; act < j1; ++act) {  // row blocks entering the band
      const uint32_t *rb = rep + 1 + 4 * act;
      const uint32_t q0 = __ldg(rb), q1 = __ldg(rb + 1), q2 = __ldg(rb + 2),
                     q3 = __ldg(rb + 3);
      const uint32_t slot = act - j0;
#pragma unroll
      for (int m = 0; m < W; ++m) {
        if ((uint32_t)m == slot) {
          P0[m] = q0;
          P1[m] = q1;
          P2[m] = q2;
          P3[m] = q3;
        }
      }
    }
    ColumnPlanes col(tar + 1 + 4 * i);
#pragma unroll 4
    for (int k = 0; k < 32; ++k) window_step<W>(V, P0, P1, P2, P3, col.next());
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

// General form for any band width: per column block the live rows are
// processed in chunks of 8 words held in `lines` (the row vector, one word per
// row block), with the 32 column carries between chunks kept as one word
// (bit k = carry of column k), like the reference's carry register.
constexpr uint32_t kMaxRowBlocks = (NGIA_MAX_READ + 31) / 32;  // 2048

__device__ inline uint32_t lcs_general(const uint32_t *__restrict__ rep,
                                const uint32_t *__restrict__ tar, const Band &b,
                                uint32_t *lines, uint32_t &blocks) {
  for (uint32_t w = 0; w < b.nr; ++w) lines[w] = kFull;
  uint32_t zeros = 0;  // running LCS: zero bits over all row blocks
  for (uint32_t i = 0; i < b.nc; ++i) {
    const uint32_t j0 = i > b.ls ? i - b.ls : 0;
    const uint32_t j1 = (i + b.rs < b.nr) ? i + b.rs : b.nr;
    const uint32_t *tb = tar + 1 + 4 * i;
    if (i > 0 && !may_reach_threshold(zeros, 32 * i, b)) {  // score 0 certain
      blocks = i;
      return 0;
    }
    uint32_t cin_word = 0;  // carries into the current chunk, bit k = column k
    for (uint32_t j = j0; j < j1; j += 8) {
      uint32_t V[8], P0[8], P1[8], P2[8], P3[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const uint32_t r = j + m;
        if (r < j1) {
          const uint32_t *rb = rep + 1 + 4 * r;
          V[m] = lines[r];
          P0[m] = __ldg(rb);
          P1[m] = __ldg(rb + 1);
          P2[m] = __ldg(rb + 2);
          P3[m] = __ldg(rb + 3);
        } else {
          V[m] = kFull;
          P0[m] = P1[m] = P2[m] = P3[m] = 0;
        }
      }
      uint32_t cout_word = 0;
      ColumnPlanes col(tb);
#pragma unroll 4
      for (int k = 0; k < 32; ++k) {
        const ColMask c = col.next();
        uint32_t t[8], s[8], co;
#pragma unroll
        for (int m = 0; m < 8; ++m) t[m] = match_and(V[m], P0[m], P1[m], P2[m], P3[m], c);
        add_chain8_cc(s, V, t, cin_word & 1u, co);
        cin_word >>= 1;
        cout_word |= co << k;
#pragma unroll
        for (int m = 0; m < 8; ++m) V[m] = s[m] | (V[m] ^ t[m]);
      }
#pragma unroll
      for (int m = 0; m < 8; ++m)
        if (j + m < j1) {
          zeros += __popc(~V[m]) - __popc(~lines[j + m]);
          lines[j + m] = V[m];
        }
      cin_word = cout_word;
    }
  }
  blocks = b.nc;
  return zeros;
}

// Width classes of the batched aligner:
//   0..10  streaming shared-memory table kernel (align_stream.cuh), one pair
//          per lane, W = 4, 5, ..., 12, 14, 16 words by stream_width (every
//          width up to 12: a window word above the band costs as much as a
//          live one, and bands of equal ls + rs - 1 are common)
//   11..18 group kernel (align_group.cuh), one pair per group of G lanes with
//          K words per lane: (8,3) (8,4) (16,4) (16,6) (32,4) (32,6) (32,8)
//          (32,16).  A column step costs a lane 3 ops per word plus a fixed
//          ~6 (carry pop and push, code, table row), and a band of span S
//          keeps about S / (K + 1) of the G lanes live, so the ladder takes
//          each span to the shape with the fewest issue slots per cell: eight
//          lanes of three or four words for the 17-36-word bands of medium
//          proteins rather than sixteen lanes of one or two
//   19     general kernel, one pair per thread (any width)
//   20     pairs failing the length filter (score 0, not launched)
constexpr int kNumLdsClasses = 11;
constexpr int kFirstGroupClass = 11;
constexpr int kNumGroupClasses = 8;
constexpr int kGeneralClass = kFirstGroupClass + kNumGroupClasses;
constexpr int kSkipClass = kGeneralClass + 1;
constexpr int kNumClasses = kSkipClass + 1;

struct GroupShape {
  int G, K;
};
__host__ __device__ constexpr GroupShape group_shape(int c) {
  return c == kFirstGroupClass ? GroupShape{8, 3}
       : c == kFirstGroupClass + 1 ? GroupShape{8, 4}
       : c == kFirstGroupClass + 2 ? GroupShape{16, 4}
       : c == kFirstGroupClass + 3 ? GroupShape{16, 6}
       : c == kFirstGroupClass + 4 ? GroupShape{32, 4}
       : c == kFirstGroupClass + 5 ? GroupShape{32, 6}
       : c == kFirstGroupClass + 6 ? GroupShape{32, 8}
                                   : GroupShape{32, 16};
}

__host__ __device__ constexpr int class_width(int c) {
  return c < 9 ? 4 + c : c == 9 ? 14 : c == 10 ? 16 : 0;
}

// Window a streaming kernel needs for a pair: the live rows of block i,
// [max(i - ls, 0), min(i + rs, nr)), inside [i - ls, i - ls + W).
__host__ __device__ inline uint32_t stream_width(const Band &b) {
  return b.ls + (b.rs < b.nr ? b.rs : b.nr);
}

// A group of G lanes with K words per lane holds at most one live slice per
// lane when the rep has at most G slices or ls + rs <= (G - 1)K + G.
__host__ __device__ inline bool group_fits(const Band &b, int G, int K) {
  const uint32_t ns = (b.nr + K - 1) / K;
  return ns <= (uint32_t)G || b.ls + b.rs <= (uint32_t)((G - 1) * K + G);
}

// Largest ls + rs a group class can hold with one live slice per lane.
__host__ __device__ constexpr uint32_t group_span_limit(int c) {
  return (uint32_t)((group_shape(c).G - 1) * group_shape(c).K + group_shape(c).G);
}

// The binning plan (what an autotuner picks): the widest window sent to the
// one-pair-per-lane kernels, and per group class the widest band (ls + rs) it
// takes (0: class unused; never above group_span_limit).  A pair goes to the
// first class that takes it; reps of at most G slices fit a group class of G
// lanes whatever the band (each slice has its own lane).
struct ClassPlan {
  uint32_t stream_max;
  uint32_t group_limit[kNumGroupClasses];
};

__host__ __device__ inline ClassPlan default_plan() {
  ClassPlan p{16, {}};
  for (int g = 0; g < kNumGroupClasses; ++g) p.group_limit[g] = group_span_limit(kFirstGroupClass + g);
  return p;
}

__host__ __device__ inline int width_class(const Band &b, const ClassPlan &plan) {
  if (!b.pass) return kSkipClass;
  const uint32_t ws = stream_width(b);
  if (ws <= plan.stream_max) return ws <= 4 ? 0 : ws <= 12 ? (int)ws - 4 : ws <= 14 ? 9 : 10;
  for (int g = 0; g < kNumGroupClasses; ++g) {
    const uint32_t lim = plan.group_limit[g];
    if (lim == 0) continue;
    const GroupShape sh = group_shape(kFirstGroupClass + g);
    const uint32_t ns = (b.nr + sh.K - 1) / sh.K;
    if (ns <= (uint32_t)sh.G || b.ls + b.rs <= lim) return kFirstGroupClass + g;
  }
  return kGeneralClass;
}

__host__ __device__ inline int width_class(const Band &b) {
  return width_class(b, default_plan());
}

// Queue order inside a class: longest targets first.  The sort key of a pair
// is class-major, then 7 - floor(log2 nc) (column blocks in octaves, capped
// at 7), one 8-bit radix pass.
__host__ __device__ inline uint32_t class_sort_key(int cls, const Band &b) {
  uint32_t h = 0;
  if (b.nc > 1) {
#ifdef __CUDA_ARCH__
    const uint32_t lg = 31u - (uint32_t)__clz(b.nc);  // floor(log2 nc)
#else
    const uint32_t lg = 31u - (uint32_t)__builtin_clz(b.nc);
#endif
    h = 2 * lg + ((uint64_t)b.nc * b.nc >= (2ull << (2 * lg)) ? 1u : 0u);
  }
  h >>= 1;
  return ((uint32_t)cls << 3) | (7u - (h < 7u ? h : 7u));
}
constexpr int kClassKeyBits = 8;
static_assert(kNumClasses <= 32, "class sort key: 5 class bits");
__host__ __device__ constexpr uint32_t skip_sort_key() { return ((uint32_t)kSkipClass << 3) | 7u; }

}  // namespace ngia
