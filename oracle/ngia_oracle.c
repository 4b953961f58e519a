/*
 * ngia_oracle.c -- CPU oracle for the group-then-align hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see ngia_oracle.h).  Compiled with
 * -ffp-contract=off so that every float operation rounds exactly where the
 * source says; the fused form is requested explicitly with fmaf().
 */
#include "ngia_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---- residue coding (src/makedb.hpp:162-171) ------------------------------
 * A reduced 15-letter alphabet; protein and nucleotide letters share it.
 * Letters not listed (X, B, Z, J, O, '*', digits, ...) code to 0, and code 0
 * matches nothing during alignment. */
uint32_t ngo_residue_code(unsigned char c) {
  switch (c | 0x20) { /* fold ASCII upper case onto lower case */
    case 'a': return 1;
    case 'c': return 2;
    case 'd': return 3;
    case 'e': case 'q': return 4;
    case 'f': case 'w': case 'y': return 5;
    case 'g': return 6;
    case 'h': return 7;
    case 'i': case 'v': return 8;
    case 'k': return 9;
    case 'l': case 'm': return 10;
    case 'n': return 11;
    case 'p': return 12;
    case 'r': return 13;
    case 's': return 14;
    case 't': case 'u': return 15;
    default: return 0;
  }
}

size_t ngo_record_words(uint32_t len) {
  return 1 + (size_t)((len + 31u) / 32u) * 4u;
}

/* Record = [len][block 0: plane0..plane3][block 1: ...]; bit r of plane e of
 * block b is bit e of the code of residue 32*b + r (src/makedb.hpp:226-231). */
void ngo_pack_record(const char *seq, uint32_t len, uint32_t *rec) {
  size_t words = ngo_record_words(len);
  memset(rec, 0, words * sizeof(uint32_t));
  rec[0] = len;
  for (uint32_t p = 0; p < len; p++) {
    uint32_t code = ngo_residue_code((unsigned char)seq[p]);
    uint32_t *blk = rec + 1 + (size_t)(p / 32u) * 4u;
    for (int e = 0; e < 4; e++) blk[e] |= ((code >> e) & 1u) << (p % 32u);
  }
}

static inline uint32_t code_at(const uint32_t *rec, uint32_t p) {
  const uint32_t *blk = rec + 1 + (size_t)(p / 32u) * 4u;
  uint32_t b = p % 32u, code = 0;
  for (int e = 0; e < 4; e++) code |= ((blk[e] >> b) & 1u) << e;
  return code;
}

/* ---- minhash sketch (src/makedb.hpp:224-248) -------------------------------
 * k-mer = the last 8 codes as one 32-bit word (newest code in the low nibble).
 * Band k hashes kmer ^ (k*0x9e3779b1 + 0x85ebca6b) with Wang's 32-bit integer
 * hash plus two extra mixing rounds and keeps the minimum.  Positions 0..6 are
 * not signed, except that a record shorter than 8 signs its last position. */
static inline uint32_t band_hash(uint32_t kmer, uint32_t band) {
  uint32_t x = kmer ^ (band * 0x9e3779b1u + 0x85ebca6bu);
  x = (x ^ 61u) ^ (x >> 16);
  x = x * 9u; /* x + (x << 3) */
  x = x ^ (x >> 4);
  x = x * 0x27d4eb2du;
  x = x ^ (x >> 15);
  x = (x ^ (x >> 8)) * 0x9e3779b1u;
  x = x ^ (x >> 14);
  return x;
}

void ngo_sketch_record(const uint32_t *rec, uint32_t sig[NGO_BANDS]) {
  uint32_t len = rec[0];
  for (int k = 0; k < NGO_BANDS; k++) sig[k] = 0xFFFFFFFFu;
  uint32_t kmer = 0;
  for (uint32_t p = 0; p < len; p++) {
    kmer = (kmer << 4) | code_at(rec, p);
    if (p < 7 && p + 1 < len) continue;
    for (uint32_t k = 0; k < NGO_BANDS; k++) {
      uint32_t h = band_hash(kmer, k);
      if (h < sig[k]) sig[k] = h;
    }
  }
}

/* ---- bucketing (src/makedb.hpp:318-348) ------------------------------------
 * The reference sorts (sig, idx) stably and links each entry to the previous
 * entry of the same signature.  The same relation, stated directly: rep[i] is
 * the largest j < i whose signature equals sig[i], or i itself.  This
 * restatement uses a hash map from signature to the last index seen. */
void ngo_bucket_band(const uint32_t *sigs, size_t stride, uint32_t n,
                     uint32_t *rep) {
  size_t cap = 16;
  while (cap < 2 * (size_t)n) cap <<= 1;
  uint32_t *keys = (uint32_t *)malloc(cap * sizeof(uint32_t));
  uint32_t *last = (uint32_t *)malloc(cap * sizeof(uint32_t));
  unsigned char *used = (unsigned char *)calloc(cap, 1);
  for (uint32_t i = 0; i < n; i++) {
    uint32_t s = sigs[(size_t)i * stride];
    size_t h = (size_t)(s * 0x9e3779b1u) & (cap - 1);
    while (used[h] && keys[h] != s) h = (h + 1) & (cap - 1);
    if (used[h]) {
      rep[i] = last[h];
    } else {
      used[h] = 1;
      keys[h] = s;
      rep[i] = i;
    }
    last[h] = i;
  }
  free(keys);
  free(last);
  free(used);
}

/* ---- band bounds (src/buildGraph.hpp:201, :208-210) -------------------------
 * t = identity / 100 in float.  A float -> uint32 conversion of a value <= 0
 * gives 0 (the GPU's saturating conversion). */
static inline float identity_threshold(uint32_t identity) {
  return (float)identity / 100.0f;
}

static inline uint32_t ceil_to_u32(float v) {
  float c = ceilf(v);
  if (!(c > 0.0f)) return 0;
  return (uint32_t)c;
}

int ngo_band_bounds(uint32_t lr, uint32_t lt, uint32_t identity, int round_mode,
                    uint32_t *lsft, uint32_t *rsft) {
  const float t = identity_threshold(identity);
  const float flr = (float)lr, flt = (float)lt;
  if (flt < flr * t) return 0;
  float dl, dr;
  if (round_mode == NGO_ROUND_FMA) {
    dl = fmaf(-flt, t, flt);
    dr = fmaf(-flt, t, flr);
  } else {
    float prod = flt * t;
    dl = flt - prod;
    dr = flr - prod;
  }
  *lsft = (ceil_to_u32(dl) + 31u) & ~31u;
  *rsft = ceil_to_u32(dr) + 32u;
  return 1;
}

static inline int32_t max_i32(int32_t a, int32_t b) { return a > b ? a : b; }
static inline int32_t min_i32(int32_t a, int32_t b) { return a < b ? a : b; }

uint64_t ngo_band_blocks(uint32_t lr, uint32_t lt, uint32_t identity,
                         int round_mode) {
  uint32_t lsft, rsft;
  if (!ngo_band_bounds(lr, lt, identity, round_mode, &lsft, &rsft)) return 0;
  uint64_t blocks = 0;
  for (int32_t i = 0; i < (int32_t)lt; i += 32) {
    int32_t js = max_i32(i - (int32_t)lsft, 0);
    int32_t je = min_i32(i + (int32_t)rsft, (int32_t)lr);
    if (je > js) blocks += (uint64_t)((je - js + 31) / 32);
  }
  return blocks;
}

/* ---- banded bit-parallel LCS (src/buildGraph.hpp:192-253) -------------------
 * Rows are the representative's residues, columns the target's.  V holds one
 * bit per row (1 = not yet matched).  For each block of 32 columns, the row
 * blocks inside the band are updated bottom to top; each column step applies
 *   V' = (V + (V & M) + carry_in) | (V & ~M)
 * where M marks rows whose code equals the column's code (code 0 matches
 * nothing) and the carry out of a row block feeds the same column of the next
 * row block.  The lowest row block of the band starts each column with carry
 * 0, and row blocks outside the band keep their value.  LCS = number of zero
 * bits over all row blocks (padding rows never clear). */
uint32_t ngo_banded_lcs(const uint32_t *rep, const uint32_t *tar,
                        uint32_t identity, int round_mode) {
  const uint32_t lr = rep[0], lt = tar[0];
  uint32_t lsft, rsft;
  if (!ngo_band_bounds(lr, lt, identity, round_mode, &lsft, &rsft)) return 0;
  const uint32_t nr = (lr + 31u) / 32u;
  uint32_t *V = (uint32_t *)malloc((nr ? nr : 1) * sizeof(uint32_t));
  for (uint32_t w = 0; w < nr; w++) V[w] = 0xFFFFFFFFu;
  for (int32_t i = 0; i < (int32_t)lt; i += 32) {
    uint32_t tcode[32];
    for (int k = 0; k < 32; k++) {
      const uint32_t *blk = tar + 1 + (size_t)(i / 32) * 4u;
      uint32_t c = 0;
      for (int e = 0; e < 4; e++) c |= ((blk[e] >> k) & 1u) << e;
      tcode[k] = c;
    }
    uint32_t cin[32];
    memset(cin, 0, sizeof(cin));
    int32_t js = max_i32(i - (int32_t)lsft, 0);
    int32_t je = min_i32(i + (int32_t)rsft, (int32_t)lr);
    for (int32_t j = js; j < je; j += 32) {
      const uint32_t *rb = rep + 1 + (size_t)(j / 32) * 4u;
      uint32_t eq[16];
      eq[0] = 0;
      for (uint32_t c = 1; c < 16; c++) {
        uint32_t m = 0xFFFFFFFFu;
        for (int e = 0; e < 4; e++) m &= ((c >> e) & 1u) ? rb[e] : ~rb[e];
        eq[c] = m;
      }
      uint32_t x = V[j / 32];
      for (int k = 0; k < 32; k++) {
        uint32_t m = eq[tcode[k]];
        uint64_t s = (uint64_t)x + (uint64_t)(x & m) + (uint64_t)cin[k];
        cin[k] = (uint32_t)(s >> 32);
        x = (uint32_t)s | (x & ~m);
      }
      V[j / 32] = x;
    }
  }
  uint32_t lcs = 0;
  for (uint32_t w = 0; w < nr; w++) lcs += 32u - (uint32_t)__builtin_popcount(V[w]);
  free(V);
  return lcs;
}

uint32_t ngo_align(const uint32_t *rep, const uint32_t *tar, uint32_t identity,
                   int round_mode) {
  const uint32_t lr = rep[0], lt = tar[0];
  uint32_t lsft, rsft;
  if (!ngo_band_bounds(lr, lt, identity, round_mode, &lsft, &rsft)) return 0;
  const float t = identity_threshold(identity);
  uint32_t lcs = ngo_banded_lcs(rep, tar, identity, round_mode);
  uint32_t den = lr + lt - lcs;
  if ((float)lcs > (float)den * t) return lcs * 100u / den;
  return 0;
}

/* ---- candidate collection (src/buildGraph.hpp:262-300) ---------------------- */
size_t ngo_collect_band(const uint32_t *rep_row, const uint32_t *lens,
                        uint32_t n, uint32_t identity, uint32_t *pairs) {
  const float t = identity_threshold(identity);
  size_t k = 0;
  for (uint32_t i = 0; i < n; i++) {
    uint32_t r = rep_row[i];
    if (r == i) continue;
    if (!((float)lens[i] >= (float)lens[r] * t)) continue;
    pairs[2 * k] = r;
    pairs[2 * k + 1] = i;
    k++;
  }
  return k;
}

void ngo_align_many(const uint32_t *packed, const uint64_t *offs,
                    const uint32_t *pairs, size_t count, uint32_t identity,
                    int round_mode, uint32_t *scores) {
  for (size_t k = 0; k < count; k++) {
    const uint32_t *rep = packed + offs[pairs[2 * k]];
    const uint32_t *tar = packed + offs[pairs[2 * k + 1]];
    scores[k] = ngo_align(rep, tar, identity, round_mode);
  }
}
