"""Seeded synthetic sequence families (stand-ins for public datasets).

Families: a root sequence drawn i.i.d. from background residue frequencies,
members derived from the root by uniform substitutions (rate drawn per member
from a range) and indels (events at a per-position rate, geometric lengths,
insertion or deletion with equal probability).  All members of all families
are shuffled with the seed.  Generation is vectorised over a chunk of
families at a time.

Workloads (sizes from the benchmark configurations):
  protein_families(20_000, 2_000, seed=1)   log-normal roots (median 300, sigma
                                            0.5, clipped 50..1500), 5-35 % subs,
                                            2 % indels of mean length 3
  dna_families(200_000, 20_000, seed=2)     uniform roots 200..3000, GC 0.45,
                                            1-10 % subs, 1 % indels of mean 2
"""
from __future__ import annotations

import numpy as np

AMINO = np.frombuffer(b"ACDEFGHIKLMNPQRSTVWY", dtype=np.uint8)
# Background amino-acid frequencies (UniProtKB/Swiss-Prot composition, %).
AMINO_FREQ = np.array([8.25, 1.37, 5.45, 6.75, 3.86, 7.07, 2.27, 5.96, 5.84, 9.66,
                       2.42, 4.06, 4.70, 3.93, 5.53, 6.56, 5.34, 6.87, 1.08, 2.92])
AMINO_FREQ = AMINO_FREQ / AMINO_FREQ.sum()
NUCLEO = np.frombuffer(b"ACGT", dtype=np.uint8)
NUCLEO_FREQ = np.array([0.275, 0.225, 0.225, 0.275])  # GC = 0.45


class SeqSet:
    """Sequences as one byte array plus lengths, in file (shuffled) order."""

    def __init__(self, residues: np.ndarray, lens: np.ndarray, names: list[bytes]):
        self.residues = residues
        self.lens = lens.astype(np.int64)
        self.names = names
        self.starts = np.concatenate([[0], np.cumsum(self.lens)[:-1]]).astype(np.int64)

    def __len__(self) -> int:
        return len(self.lens)

    def seq(self, i: int) -> bytes:
        s = int(self.starts[i])
        return self.residues[s:s + int(self.lens[i])].tobytes()

    def fasta_bytes(self, line_width: int = 0) -> bytes:
        out = []
        for i in range(len(self)):
            out.append(self.names[i])
            out.append(b"\n")
            s = self.seq(i)
            if line_width and len(s) > line_width:
                for k in range(0, len(s), line_width):
                    out.append(s[k:k + line_width])
                    out.append(b"\n")
            else:
                out.append(s)
                out.append(b"\n")
        return b"".join(out)

    def write_fasta(self, path, line_width: int = 0) -> None:
        with open(path, "wb") as f:
            f.write(self.fasta_bytes(line_width))


def _draw(rng, alphabet, freqs, k):
    """k residues i.i.d. from the background frequencies."""
    cdf = np.cumsum(freqs)
    cdf[-1] = 1.0
    u = rng.random(k, dtype=np.float32)
    return alphabet[np.minimum(np.searchsorted(cdf, u, side="right"), len(alphabet) - 1)]


def _mutate_chunk(rng, roots, root_lens, per_family, alphabet, freqs, sub_lo, sub_hi,
                  indel_rate, indel_mean):
    """Members of a chunk of families; returns (residues, lens, family ids)."""
    fam = np.repeat(np.arange(len(root_lens)), per_family)
    mlen = root_lens[fam]
    root_start = np.concatenate([[0], np.cumsum(root_lens)[:-1]])
    total = int(mlen.sum())
    member_of = np.repeat(np.arange(len(fam)), mlen)
    member_start = np.concatenate([[0], np.cumsum(mlen)[:-1]])
    pos_in = np.arange(total) - member_start[member_of]
    base = roots[root_start[fam][member_of] + pos_in]
    # substitutions
    rate = rng.uniform(sub_lo, sub_hi, size=len(fam)).astype(np.float32)
    sub = rng.random(total, dtype=np.float32) < rate[member_of]
    base[sub] = _draw(rng, alphabet, freqs, int(sub.sum()))
    # indel events
    ev = np.flatnonzero(rng.random(total, dtype=np.float32) < indel_rate)
    is_del = rng.random(len(ev)) < 0.5
    length = rng.geometric(1.0 / indel_mean, size=len(ev))
    member_end = (member_start + mlen)[member_of]
    # deletions: positions [p, min(p + len, member end))
    dels, dlen = ev[is_del], length[is_del]
    dend = np.minimum(dels + dlen, member_end[dels])
    cover = (np.bincount(dels, minlength=total + 1)
             - np.bincount(dend, minlength=total + 1)).astype(np.int32)
    keep = np.cumsum(cover[:-1]) == 0
    # insertions: `len` random residues before position p
    ins_len = np.bincount(ev[~is_del], weights=length[~is_del],
                          minlength=total).astype(np.int64)
    out_count = ins_len + keep
    src = np.repeat(np.arange(total), out_count)
    group_start = np.concatenate([[0], np.cumsum(out_count)[:-1]])
    rank = np.arange(len(src)) - group_start[src]
    inserted = rank < ins_len[src]
    out = base[src]
    n_ins = int(inserted.sum())
    if n_ins:
        out[inserted] = _draw(rng, alphabet, freqs, n_ins)
    new_lens = np.bincount(member_of[src], minlength=len(fam))
    return out, new_lens, fam


def families(n_seqs, n_families, alphabet, freqs, root_len_fn, sub_lo, sub_hi, indel_rate,
             indel_mean, seed, chunk_families=2000, prefix=b"fam") -> SeqSet:
    rng = np.random.default_rng(seed)
    per = np.full(n_families, n_seqs // n_families, dtype=np.int64)
    per[: n_seqs - int(per.sum())] += 1
    res_parts, len_parts, fam_parts, mem_parts = [], [], [], []
    for f0 in range(0, n_families, chunk_families):
        f1 = min(n_families, f0 + chunk_families)
        rl = root_len_fn(rng, f1 - f0).astype(np.int64)
        roots = _draw(rng, alphabet, freqs, int(rl.sum()))
        out, lens, fam = _mutate_chunk(rng, roots, rl, per[f0:f1], alphabet, freqs, sub_lo,
                                       sub_hi, indel_rate, indel_mean)
        res_parts.append(out)
        len_parts.append(lens)
        fam_parts.append(fam + f0)
        mem_parts.append(np.concatenate([np.arange(k) for k in per[f0:f1]]))
    residues = np.concatenate(res_parts)
    lens = np.concatenate(len_parts)
    fam = np.concatenate(fam_parts)
    mem = np.concatenate(mem_parts)
    order = rng.permutation(len(lens))
    starts = np.concatenate([[0], np.cumsum(lens)[:-1]])
    # gather the shuffled order into one array
    idx = np.concatenate([np.arange(starts[i], starts[i] + lens[i]) for i in order]) \
        if len(order) < 2000 else _gather_runs(starts[order], lens[order])
    names = [b">%s%06d_%02d" % (prefix, fam[i], mem[i]) for i in order]
    return SeqSet(residues[idx], lens[order], names)


def _gather_runs(starts, lens):
    total = int(lens.sum())
    run_start = np.concatenate([[0], np.cumsum(lens)[:-1]])
    owner = np.repeat(np.arange(len(lens)), lens)
    return starts[owner] + (np.arange(total) - run_start[owner])


def _lognormal_roots(median, sigma, lo, hi):
    def fn(rng, k):
        return np.clip(np.round(rng.lognormal(np.log(median), sigma, size=k)), lo, hi)
    return fn


def _uniform_roots(lo, hi):
    def fn(rng, k):
        return rng.integers(lo, hi + 1, size=k)
    return fn


def protein_families(n_seqs=20_000, n_families=2_000, seed=1) -> SeqSet:
    return families(n_seqs, n_families, AMINO, AMINO_FREQ, _lognormal_roots(300, 0.5, 50, 1500),
                    0.05, 0.35, 0.02, 3.0, seed, prefix=b"prot")


def dna_families(n_seqs=200_000, n_families=20_000, seed=2) -> SeqSet:
    return families(n_seqs, n_families, NUCLEO, NUCLEO_FREQ, _uniform_roots(200, 3000),
                    0.01, 0.10, 0.01, 2.0, seed, prefix=b"dna")
