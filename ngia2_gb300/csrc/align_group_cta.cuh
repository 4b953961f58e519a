// align_group_cta.cuh -- the group aligner with one block of W warps per pair
// (G = 32W lanes), for the widest bands (internal header).
//
// Same slices, skewed steps, band edges, tables and early exit as
// align_group.cuh; what changes is the group's size.  A lane's column step
// costs a carry chain of K words, and one warp issues one instruction a
// cycle, so a pair of a few thousand column blocks on one warp takes as long
// as its K-word chains in series: the widest classes, whose few longest pairs
// make the end of a round, ran on few warps with the SM mostly waiting.  Here
// the same band is cut into W times as many slices of K/W words: each lane's
// chain is W times shorter and a pair's steps run on W warps at once.
//
// Lanes exchange through shared memory at warp boundaries: lane 31 of warp w
// publishes its carries and slice index at the end of a step, lane 0 of warp
// w + 1 (ring) takes them after the step's barrier (two buffers by step
// parity, so one barrier a step).  Every fourth step the bound's sums, maxima
// and the ring-order suffix scan by rank go through per-warp partials in
// shared memory (three more barriers).  The block claims its pairs from the
// class's queue one at a time.
//
// Binning is unchanged: a class of (32 lanes, K words) runs here as (32W
// lanes, K/W words): the same rows per ring turn (32K), and a wider slice-free
// span, (32W - 1)K/W + 32W >= 31K + 32, so every pair the class takes keeps
// one live slice per lane.
#pragma once

#include "align_group.cuh"

namespace ngia {

template <int W>
struct CtaExchange {
  uint32_t pub_c[2][W], pub_q[2][W];  // lane 31 of each warp, by step parity
  uint32_t wsum[W], wmax[W], wzero[W], wlow[W], wbest[W];
  uint32_t qall[32 * W], sufw[32 * W];
  uint32_t claim;
};

template <int W, int K, int KC>
__host__ __device__ constexpr size_t group_cta_smem_bytes() {
  return (size_t)W * 32 * KC * K * 4 + sizeof(CtaExchange<W>);
}

// The persistent kernel body: the block takes pairs from order[begin, end)
// through `cursor`, one at a time.  Returns the lane's computed
// (word x column block) count.
template <int W, int K, int KC>
__device__ inline uint32_t align_group_cta(const uint32_t *__restrict__ packed,
                                           const uint32_t *__restrict__ nib, uint64_t inv,
                                           const uint64_t *__restrict__ offs,
                                           const uint2 *__restrict__ pairs,
                                           const uint32_t *__restrict__ order, uint32_t begin,
                                           uint32_t end, unsigned int *__restrict__ cursor,
                                           uint32_t *__restrict__ scores, float t, int fma_mode,
                                           uint32_t *smem) {
  constexpr uint32_t G = 32u * W;
  constexpr uint32_t kNone = 0xFFFFFFFFu;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t sub = threadIdx.x;  // the lane's place in the group
  const LdsTable<K, KC> tab{smem + warp * (KC * K * 32) + lane, inv};
  CtaExchange<W> &xc = *reinterpret_cast<CtaExchange<W> *>(smem + W * KC * K * 32);
#pragma unroll 1
  for (uint32_t s = 0; s < (uint32_t)K; ++s) {
    tab.clear(s);
    tab.slot(s)[0] = 0u;
  }
  uint32_t V[K];
#pragma unroll
  for (int m = 0; m < K; ++m) V[m] = kFull;

  bool active = false;
  const uint32_t *rep = nullptr, *tar = nullptr;
  uint32_t p = 0, lr = 0, lt = 0, ls = 0, rs = 0, nr = 0, nc = 0, ns = 0, tau = 0, tau_end = 0;
  uint32_t q = 0, e = 0, r = 0, zret = 0, pub_q = kNoSlice, pub_c = 0;
  uint4 codes = make_uint4(0u, 0u, 0u, 0u);
  uint4 nxt = codes, pf = codes;
  uint32_t nxt_q = kNoSlice, nxt_i = 0, pf_row = kFull;
  uint32_t done = 0, wstep = 0, parity = 0;

  for (;;) {
    if (!active) {  // block-uniform: the next pair of the class
      __syncthreads();
      if (threadIdx.x == 0) {
        const uint32_t k = begin + atomicAdd(cursor, 1u);
        xc.claim = k < end ? order[k] : kNone;
      }
      __syncthreads();
      const uint32_t pk = xc.claim;
      if (pk == kNone) break;
      p = pk;
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
      const uint32_t top = nc + rs - 1 < nr ? nc + rs - 1 : nr;
      ns = (top + K - 1) / K;
      if (nc == 0 || ns == 0) {
        if (sub == 0) scores[p] = identity_score(0u, lr, lt, t);
        continue;
      }
      active = true;
      tau = 0;
      tau_end = nc + ns - 1;
      q = sub;
      e = r = zret = 0;
      pub_q = kNoSlice;
      pub_c = 0;
      nxt_q = kNoSlice;
      pf_row = kFull;
      wstep = 0;
      if (lane == 31) {  // nothing crosses a warp boundary into the first step
        xc.pub_c[parity][warp] = 0u;
        xc.pub_q[parity][warp] = kNoSlice;
      }
    }
    __syncthreads();  // the previous step's boundary carries are published
    uint32_t cin = __shfl_sync(kFull, pub_c, (lane + 31u) & 31u);
    uint32_t qin = __shfl_sync(kFull, pub_q, (lane + 31u) & 31u);
    if (lane == 0) {
      const uint32_t wb = (warp + W - 1) % W;
      cin = xc.pub_c[parity][wb];
      qin = xc.pub_q[parity][wb];
    }
    bool live = false;
    uint32_t I = 0;
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
        if (I + 1 < nc) {
          const uint32_t j1n = I + 1 + rs < nr ? I + 1 + rs : nr;
          if (e < (uint32_t)K && lo + e < j1n && pf_row != lo + e) {
            pf_row = lo + e;
            pf = load4(rep + 1 + 4 * pf_row);
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
    parity ^= 1u;
    if (lane == 31) {
      xc.pub_c[parity][warp] = pub_c;
      xc.pub_q[parity][warp] = pub_q;
    }

    // bound of the final LCS every fourth step, and the end of the pair
    // (block-uniform: every lane holds the same tau)
    ++wstep;
    const bool last = tau + 1 >= tau_end;
    const bool check = (wstep & 3u) == 0 || last;
    uint32_t S = 0, qhi1 = 0, ub = 0;
    if (check) {
      uint32_t livez = 0;
#pragma unroll
      for (int m = 0; m < K; ++m) livez += __popc(~V[m]);
      // within the warp: sums, the max, and the suffix sums of live zeros
      uint32_t ws = zret + livez, wm = (q < ns && e > 0) ? q + 1 : 0u, suf = livez;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ws += __shfl_xor_sync(kFull, ws, o);
        wm = max(wm, __shfl_xor_sync(kFull, wm, o));
      }
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_down_sync(kFull, suf, o);
        if (lane + o < 32) suf += v;
      }
      const uint32_t wz = __shfl_sync(kFull, suf, 0);  // the warp's live zeros
      if (lane == 0) {
        xc.wsum[warp] = ws;
        xc.wmax[warp] = wm;
        xc.wzero[warp] = wz;
      }
      xc.qall[sub] = q;
      xc.sufw[sub] = suf;
      __syncthreads();
      uint32_t T = 0, after = 0;  // live zeros of all lanes, of the warps above mine
#pragma unroll
      for (int w = 0; w < W; ++w) {
        S += xc.wsum[w];
        qhi1 = max(qhi1, xc.wmax[w]);
        T += xc.wzero[w];
        if ((uint32_t)w > warp) after += xc.wzero[w];
      }
      // the lowest slice: its ring neighbour below does not hold q - 1
      const bool lowest = xc.qall[(sub + G - 1) % G] != q - 1u;
      const uint32_t lowbits = __ballot_sync(kFull, lowest);
      if (lane == 0) xc.wlow[warp] = lowbits;
      __syncthreads();
      uint32_t low = 0;
#pragma unroll
      for (int w = W - 1; w >= 0; --w)
        if (xc.wlow[w]) low = 32u * w + (uint32_t)(__ffs(xc.wlow[w]) - 1);
      // zeros of the live words of slices at or above this one in ring order
      // from the lowest: suffix sums in lane order, rotated by `low`
      uint32_t suf_low = xc.sufw[low];
#pragma unroll
      for (int w = 0; w < W; ++w)
        if ((uint32_t)w > low / 32u) suf_low += xc.wzero[w];
      const uint32_t mine = suf + after;
      const uint32_t above = sub >= low ? mine + T - suf_low : mine - suf_low;
      const uint32_t ref = qhi1 && qhi1 <= tau + 1 ? tau + 1 - qhi1 : 0u;
      const uint32_t cols = 32 * ref < lt ? 32 * ref : lt;
      const uint32_t left = lt - cols;
      uint32_t acc = S - above;
      uint32_t best = sub == low ? acc + min(left, lr) : 0u;
      const uint32_t row0 = 32u * K * q;
#pragma unroll
      for (int m = 0; m < K; ++m) {
        acc += __popc(~V[m]);
        const uint32_t row = row0 + 32u * m;
        best = max(best, acc + min(left, lr > row ? lr - row : 0u));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(kFull, best, o));
      if (lane == 0) xc.wbest[warp] = best;
      __syncthreads();
#pragma unroll
      for (int w = 0; w < W; ++w) ub = max(ub, xc.wbest[w]);
    }
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
  return done;
}

}  // namespace ngia
