/*
 * ngia_oracle.h -- CPU oracle for the group-then-align hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference's arithmetic, used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py as the checker.  No product code path links,
 * loads or calls it.
 *
 * Each function cites the reference source (SIAT-HPCC/nGIA2, src/...) whose
 * behaviour it restates.  Parity of this restatement is pinned against the
 * reference itself: tests/golden/ holds outputs of the reference's own
 * makedb / alignment / Leiden code built as a CPU program (oracle/ref_build.sh)
 * and tests/test_oracle.py checks this file against them.
 */
#ifndef NGIA_ORACLE_H
#define NGIA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NGO_BANDS 64

/* Band-bound arithmetic variants for ceil(L - Lt*t):
 *   NGO_ROUND_SPLIT : product rounded to float, then subtracted (two roundings)
 *   NGO_ROUND_FMA   : fused multiply-add (one rounding), the form a GPU build
 *                     with multiply-add contraction produces. */
#define NGO_ROUND_SPLIT 0
#define NGO_ROUND_FMA 1

/* 4-bit residue code (src/makedb.hpp:162-171). */
uint32_t ngo_residue_code(unsigned char c);

/* Words in a packed record [len][4*ceil(len/32) plane words]
 * (src/makedb.hpp:15-17, :142, :223). */
size_t ngo_record_words(uint32_t len);

/* Pack one residue string into a record (src/makedb.hpp:222-231). */
void ngo_pack_record(const char *seq, uint32_t len, uint32_t *rec);

/* 64 minhash signatures of one packed record (src/makedb.hpp:224-248). */
void ngo_sketch_record(const uint32_t *rec, uint32_t sig[NGO_BANDS]);

/* Bucket one band: rep[i] = largest j < i with sig[j] == sig[i], else i.
 * sig[i] is read at sigs[i * stride]
 * (src/makedb.hpp:318-348: stable sort by (sig, idx) + predecessor chain). */
void ngo_bucket_band(const uint32_t *sigs, size_t stride, uint32_t n,
                     uint32_t *rep);

/* Band bounds of the banded alignment (src/buildGraph.hpp:208-210).
 * Returns 0 when the pair fails the length filter (src/buildGraph.hpp:201),
 * else 1 and fills lsft, rsft (residue units, as in the reference). */
int ngo_band_bounds(uint32_t lr, uint32_t lt, uint32_t identity, int round_mode,
                    uint32_t *lsft, uint32_t *rsft);

/* Identity score of one pair, exactly as kernel_dynamic computes it
 * (src/buildGraph.hpp:192-253).  rep/tar point at packed records. */
uint32_t ngo_align(const uint32_t *rep, const uint32_t *tar, uint32_t identity,
                   int round_mode);

/* LCS value of the banded computation (same as above, before scoring). */
uint32_t ngo_banded_lcs(const uint32_t *rep, const uint32_t *tar,
                        uint32_t identity, int round_mode);

/* Number of 32x32 blocks the reference loop visits for a pair
 * (0 when the length filter rejects it).  Aligned cells = 1024 * blocks. */
uint64_t ngo_band_blocks(uint32_t lr, uint32_t lt, uint32_t identity,
                         int round_mode);

/* Candidate pairs of one band in index order (src/buildGraph.hpp:262-300):
 * i with rep[i] != i and len[i] >= len[rep[i]] * t.  Writes (rep, tar) to
 * pairs[2k], pairs[2k+1]; returns the count. */
size_t ngo_collect_band(const uint32_t *rep_row, const uint32_t *lens,
                        uint32_t n, uint32_t identity, uint32_t *pairs);

/* Score many pairs.  packed = packed region as u32 words, offs = word offset
 * of each record, pairs = (rep, tar) u32 pairs; scores[k] written. */
void ngo_align_many(const uint32_t *packed, const uint64_t *offs,
                    const uint32_t *pairs, size_t count, uint32_t identity,
                    int round_mode, uint32_t *scores);

#ifdef __cplusplus
}
#endif
#endif
