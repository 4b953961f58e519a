// align_group.cuh -- banded bit-parallel LCS of one pair by a group of G
// lanes, for bands wider than a thread's window (internal header).
//
// Same recurrence, match tables and column steps as align_lds.cuh; the band's
// row words are spread over the lanes of a group.
//
// Slices.  The rep's row words are cut into slices of K consecutive words;
// slice q belongs to lane q % G of the group, which takes its slices in
// increasing order (its table and its K words of V are reused for slice
// q + G once slice q is finished).
//
// Skewed steps.  Slice q handles column block I at group step tau = I + q.
// It needs its own words after block I - 1 (its lane's step tau - 1) and the
// 32 carries that leave slice q - 1's top word during block I (the lane below,
// step tau - 1).  So each step a lane runs the 32 column steps of one column
// block over its K words with the carries of the lane below, and hands its
// own 32 carries up one lane with a shuffle.  The carries travel as a word:
// the producing chain appends each column's carry at the bottom
// (addc x, x, x), the consuming chain pops them from the top (add.cc x, x, x)
// straight into the carry flag of its first word (carry_chain.cuh).
//
// Band edges.  Words below J0(I) are frozen in the reference: here they are
// counted, reset to all ones and their table entries cleared, after which
// they pass a carry through unchanged -- the carry into J0 is then whatever
// enters the slice, which is 0 because the slice below is finished (its lane
// has moved on, so the carry is not taken).  Words at or above J1(I) have not
// entered: all ones with zero masks, the reference's unvisited rows.
//
// One live slice per lane.  Slice q is live at step tau when
// q(K+1) lies in (tau - ls - K, tau + rs); slices q and q + G are never live
// together when ls + rs <= (G - 1)K + G, or when the rep has at most G
// slices.  Pairs are binned so that one of the two holds.
//
// Early exit.  With a zero carry into the band's lowest row, a column step
// never lowers the number of zeros below any row, and the total rises by at
// most one per column.  Let qhi be the highest slice with rows in the band and
// c the column where slice qhi + 1 stands (one block behind qhi): at c no row
// above slice qhi is in the band, so the zeros of the slices through any row
// j, each counted after its own latest block, bound the banded LCS through
// row j at c (the slices below run ahead).  (At qhi's own column that fails:
// rows of the slices above may be in the band there uncounted -- at a pair's
// first block every row word below rs.)  The final LCS then stays within
//   max over rows j of  zeros through j + min(columns after c, Lr - j),
// taken per word (zeros through its last row, rows above its first) plus the
// retired rows' term; once that fails the identity test the score is 0.
#pragma once

#include "align_lds.cuh"

namespace ngia {

constexpr int kGroupThreads = 64;  // threads per block (each warp owns its tables)
constexpr uint32_t kNoSlice = 0xFFFFFFFFu;

__host__ __device__ constexpr size_t group_smem_bytes(int K, int KC) {
  return (size_t)kGroupThreads * KC * K * 4;
}

// Lanes that lead a group of G (lane % G == 0).
template <int G>
__host__ __device__ constexpr uint32_t group_leaders() {
  uint32_t m = 0;
  for (int l = 0; l < 32; l += G) m |= 1u << l;
  return m;
}

// 32 column steps of one column block over the lane's K words.
template <int K>
__device__ __forceinline__ void group_columns(uint32_t (&V)[K], const uint32_t *tab,
                                              const uint4 &nib, uint32_t cin,
                                              uint32_t &cout) {
  uint32_t w0 = nib.x, w1 = nib.y, w2 = nib.z, w3 = nib.w;
  cout = 0;
#pragma unroll 1
  for (int q = 0; q < 4; ++q) {
    uint32_t x = w0;
    w0 = w1;
    w1 = w2;
    w2 = w3;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      uint32_t code;
      asm("mul.hi.u32 %0, %1, 16;" : "=r"(code) : "r"(x));
      asm("mul.lo.u32 %0, %0, 16;" : "+r"(x));
      const uint32_t *row = tab + code * (K * 32);
      uint32_t t[K], s[K];
#pragma unroll
      for (int m = 0; m < K; ++m) t[m] = V[m] & row[m * 32];
      add_words_pp<K>(s, V, t, cin, cout);
#pragma unroll
      for (int m = 0; m < K; ++m) V[m] = s[m] | (V[m] ^ t[m]);
    }
  }
}

template <int G>
__device__ __forceinline__ uint32_t group_sum(uint32_t v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

template <int G>
__device__ __forceinline__ uint32_t group_max(uint32_t v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// The early-exit bound of the group's pair (every lane of the warp calls it;
// the values of groups without a pair are never used).  The lanes hold G
// consecutive slices, slice q in lane q % G: the lowest is the one whose ring
// neighbour below does not hold q - 1, and a lane's rank is its distance
// above it.  Suffix sums of the live zeros by rank give each lane the zeros of
// every row below its slice (S holds all of them plus the retired rows'), and
// each of its words bounds the LCS through its rows plus min(left, rows above
// its first row); the lowest lane adds the retired rows' term.
template <int G, int K>
__device__ __forceinline__ uint32_t group_row_bound(const uint32_t (&V)[K], uint32_t q,
                                                    uint32_t lane, uint32_t sub, uint32_t src,
                                                    uint32_t S, uint32_t live, uint32_t left,
                                                    uint32_t lr) {
  constexpr uint32_t kGroupBits = G == 32 ? kFull : (1u << G) - 1u;
  const bool lowest = __shfl_sync(kFull, q, src) != q - 1u;
  const uint32_t bits = (__ballot_sync(kFull, lowest) >> (lane - sub)) & kGroupBits;
  const uint32_t low = (uint32_t)(__ffs(bits) - 1) & (uint32_t)(G - 1);
  const uint32_t rank = (sub + G - low) % G;
  uint32_t above = live;  // live zeros of this slice and the ones above it
#pragma unroll
  for (int o = 1; o < G; o <<= 1) {
    const uint32_t v = __shfl_sync(kFull, above, lane - sub + (sub + o) % G);
    if (rank + o < (uint32_t)G) above += v;
  }
  uint32_t acc = S - above;
  uint32_t best = rank == 0 ? acc + min(left, lr) : 0u;
  const uint32_t row0 = 32u * K * q;
#pragma unroll
  for (int m = 0; m < K; ++m) {
    acc += __popc(~V[m]);
    const uint32_t row = row0 + 32u * m;
    best = max(best, acc + min(left, lr > row ? lr - row : 0u));
  }
  return group_max<G>(best);
}

// The persistent kernel body of one group class: groups take pairs from
// order[begin, end) through `cursor`.  Returns the lane's computed
// (word x column block) count.
template <int G, int K, int KC>
__device__ inline uint32_t align_group(const uint32_t *__restrict__ packed,
                                       const uint32_t *__restrict__ nib, uint64_t inv,
                                       const uint64_t *__restrict__ offs,
                                       const uint2 *__restrict__ pairs,
                                       const uint32_t *__restrict__ order, uint32_t begin,
                                       uint32_t end, unsigned int *__restrict__ cursor,
                                       uint32_t *__restrict__ scores, float t, int fma_mode,
                                       uint32_t *smem) {
  static_assert(G == 8 || G == 16 || G == 32, "groups of 8, 16 or 32 lanes");
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t sub = lane % G;
  const uint32_t src = lane - sub + (sub + G - 1) % G;  // the lane below in the ring
  const LdsTable<K, KC> tab{smem + (threadIdx.x >> 5) * (KC * K * 32) + lane, inv};
#pragma unroll 1
  for (uint32_t s = 0; s < (uint32_t)K; ++s) {
    tab.clear(s);
    tab.slot(s)[0] = 0u;
  }
  uint32_t V[K];
#pragma unroll
  for (int m = 0; m < K; ++m) V[m] = kFull;

  // the group's pair (same in all its lanes)
  bool active = false, drained = false;
  const uint32_t *rep = nullptr, *tar = nullptr;
  uint32_t p = 0, lr = 0, lt = 0, ls = 0, rs = 0, nr = 0, nc = 0, ns = 0, tau = 0, tau_end = 0;
  // this lane's slice
  uint32_t q = 0, e = 0, r = 0, zret = 0, pub_q = kNoSlice, pub_c = 0;
  uint4 codes = make_uint4(0u, 0u, 0u, 0u);
  // loads issued one step ahead: the slice's next code block, the planes of
  // its next entering word
  uint4 nxt = codes, pf = codes;
  uint32_t nxt_q = kNoSlice, nxt_i = 0, pf_row = kFull;
  uint32_t done = 0, wstep = 0;

  for (;;) {
    // groups without a pair take the next ones (one atomic per warp)
    const uint32_t need = __ballot_sync(kFull, !active && !drained) & group_leaders<G>();
    if (need) {
      const uint32_t leader = __ffs(need) - 1;
      uint32_t first = 0;
      if (lane == leader) first = atomicAdd(cursor, (unsigned int)__popc(need));
      first = __shfl_sync(kFull, first, leader);
      if (!active && !drained) {
        const uint32_t k = begin + first + __popc(need & ((1u << (lane - sub)) - 1u));
        if (k < end) {
          p = order[k];
          const uint2 pr = pairs[p];
          const uint64_t to = offs[pr.y];
          rep = packed + offs[pr.x];
          tar = nib + to + 1;
          lr = __ldg(rep);
          lt = __ldg(packed + to);
          const Band b = make_band(lr, lt, t, fma_mode);
          ls = b.ls;
          rs = b.rs;
          nr = b.nr;
          nc = b.nc;
          // rows at or above J1 of the last column block never enter the band
          const uint32_t top = nc + rs - 1 < nr ? nc + rs - 1 : nr;
          ns = (top + K - 1) / K;
          if (nc == 0 || ns == 0) {
            if (sub == 0) scores[p] = identity_score(0u, lr, lt, t);
          } else {
            active = true;
            tau = 0;
            tau_end = nc + ns - 1;
            q = sub;
            e = r = zret = 0;
            pub_q = kNoSlice;
            pub_c = 0;
            nxt_q = kNoSlice;
            pf_row = kFull;
          }
        } else {
          drained = true;
        }
      }
    }
    if (!__any_sync(kFull, active)) {
      if (__all_sync(kFull, drained)) break;
      continue;
    }

    // carries of the previous step from the lane below
    uint32_t cin = __shfl_sync(kFull, pub_c, src);
    const uint32_t qin = __shfl_sync(kFull, pub_q, src);
    bool live = false;
    uint32_t I = 0;
    if (active) {
      // move past finished slices (all words below J0, or every column done)
      while (q < ns && tau >= q) {
        I = tau - q;
        const uint32_t j0 = I > ls ? I - ls : 0u;
        if (I < nc && (q + 1) * K > j0) break;
#pragma unroll
        for (int m = 0; m < K; ++m) {
          zret += __popc(~V[m]);
          V[m] = kFull;
        }
#pragma unroll 1
        for (uint32_t s = 0; s < (uint32_t)K; ++s) tab.clear(s);
        e = r = 0;
        q += G;
      }
      if (q < ns && tau >= q) {
        I = tau - q;
        const uint32_t j0 = I > ls ? I - ls : 0u;
        const uint32_t j1 = I + rs < nr ? I + rs : nr;
        const uint32_t lo = q * K;
        if (lo < j1) {
          live = true;
          const uint32_t rr = j0 > lo ? (j0 - lo < (uint32_t)K ? j0 - lo : (uint32_t)K) : 0u;
          if (rr > r) {  // words leaving the band
#pragma unroll
            for (int m = 0; m < K; ++m)
              if ((uint32_t)m >= r && (uint32_t)m < rr) {
                zret += __popc(~V[m]);
                V[m] = kFull;
                tab.clear(m);
              }
            r = rr;
          }
          const uint32_t ee = j1 - lo < (uint32_t)K ? j1 - lo : (uint32_t)K;
          for (; e < ee; ++e)
            tab.fill(e, lo + e == pf_row ? pf : load4(rep + 1 + 4 * (lo + e)));
          // next step's loads: this slice's next code block and the word
          // that enters then (J1 moves up at most one word per block)
          if (I + 1 < nc) {
            const uint32_t j1n = I + 1 + rs < nr ? I + 1 + rs : nr;
            if (e < (uint32_t)K && lo + e < j1n && pf_row != lo + e) {
              pf_row = lo + e;
              pf = load4(rep + 1 + 4 * pf_row);
            }
          }
        }
      }
    }
    cin = (live && q > 0 && qin == q - 1) ? cin : 0u;
    uint32_t cout = 0;
    if (live) {
      codes = (nxt_q == q && nxt_i == I) ? nxt : load4(tar + 4 * I);
      if (I + 1 < nc) {
        nxt = load4(tar + 4 * (I + 1));
        nxt_q = q;
        nxt_i = I + 1;
      }
      group_columns<K>(V, tab.base, codes, cin, cout);
      done += K;
    }
    pub_c = cout;
    pub_q = live ? q : kNoSlice;

    // bound of the final LCS every fourth step, and the end of the pair
    ++wstep;
    const bool last = active && tau + 1 >= tau_end;
    const bool check = (wstep & 3u) == 0 || __any_sync(kFull, last);
    uint32_t S = 0, qhi1 = 0, ub = 0;
    if (check) {
      uint32_t live = 0;
#pragma unroll
      for (int m = 0; m < K; ++m) live += __popc(~V[m]);
      S = group_sum<G>(zret + live);
      qhi1 = group_max<G>((active && q < ns && e > 0) ? q + 1 : 0u);
      // column blocks done where slice qhi + 1 stands (qhi + 1 <= tau + 1)
      const uint32_t ref = qhi1 && qhi1 <= tau + 1 ? tau + 1 - qhi1 : 0u;
      const uint32_t cols = 32 * ref < lt ? 32 * ref : lt;
      ub = group_row_bound<G, K>(V, q, lane, sub, src, S, live, lt - cols, lr);
    }
    if (active) {
      ++tau;
      bool fin = tau >= tau_end;
      uint32_t score = 0;
      if (fin) {
        score = identity_score(S, lr, lt, t);
      } else if (check && qhi1) {
        fin = !lcs_may_reach(ub, lr, lt, t);
      }
      if (fin) {
        if (sub == 0) scores[p] = score;
        active = false;
#pragma unroll
        for (int m = 0; m < K; ++m) V[m] = kFull;
#pragma unroll 1
        for (uint32_t s = 0; s < (uint32_t)K; ++s) tab.clear(s);
        pub_q = kNoSlice;
        pub_c = 0;
      }
    }
  }
  return done;
}

}  // namespace ngia
