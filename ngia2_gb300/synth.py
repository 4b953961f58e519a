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
                  indel_rate, indel_mean, with_root=False):
    """Members of a chunk of families; returns (residues, lens, family ids).
    with_root: member 0 of every family is the root itself."""
    fam = np.repeat(np.arange(len(root_lens)), per_family)
    mlen = root_lens[fam]
    root_start = np.concatenate([[0], np.cumsum(root_lens)[:-1]])
    total = int(mlen.sum())
    member_of = np.repeat(np.arange(len(fam)), mlen)
    member_start = np.concatenate([[0], np.cumsum(mlen)[:-1]])
    pos_in = np.arange(total) - member_start[member_of]
    base = roots[root_start[fam][member_of] + pos_in]
    first = np.concatenate([[True], fam[1:] != fam[:-1]])  # member 0 of each family
    # substitutions
    rate = rng.uniform(sub_lo, sub_hi, size=len(fam)).astype(np.float32)
    ind = np.full(len(fam), indel_rate, dtype=np.float32)
    if with_root:
        rate[first] = 0.0
        ind[first] = 0.0
    sub = rng.random(total, dtype=np.float32) < rate[member_of]
    base[sub] = _draw(rng, alphabet, freqs, int(sub.sum()))
    # indel events
    ev = np.flatnonzero(rng.random(total, dtype=np.float32) < ind[member_of])
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
             indel_mean, seed, chunk_families=2000, prefix=b"fam",
             with_root=False) -> SeqSet:
    rng = np.random.default_rng(seed)
    per = np.full(n_families, n_seqs // n_families, dtype=np.int64)
    per[: n_seqs - int(per.sum())] += 1
    res_parts, len_parts, fam_parts, mem_parts = [], [], [], []
    for f0 in range(0, n_families, chunk_families):
        f1 = min(n_families, f0 + chunk_families)
        rl = root_len_fn(rng, f1 - f0).astype(np.int64)
        roots = _draw(rng, alphabet, freqs, int(rl.sum()))
        out, lens, fam = _mutate_chunk(rng, roots, rl, per[f0:f1], alphabet, freqs, sub_lo,
                                       sub_hi, indel_rate, indel_mean, with_root)
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


class _LogNormalRoots:  # classes rather than closures: they pickle into workers
    def __init__(self, median, sigma, lo, hi):
        self.median, self.sigma, self.lo, self.hi = median, sigma, lo, hi

    def __call__(self, rng, k):
        return np.clip(np.round(rng.lognormal(np.log(self.median), self.sigma, size=k)),
                       self.lo, self.hi)


class _UniformRoots:
    def __init__(self, lo, hi):
        self.lo, self.hi = lo, hi

    def __call__(self, rng, k):
        return rng.integers(self.lo, self.hi + 1, size=k)


def _lognormal_roots(median, sigma, lo, hi):
    return _LogNormalRoots(median, sigma, lo, hi)


def _uniform_roots(lo, hi):
    return _UniformRoots(lo, hi)


def protein_families(n_seqs=20_000, n_families=2_000, seed=1) -> SeqSet:
    return families(n_seqs, n_families, AMINO, AMINO_FREQ, _lognormal_roots(300, 0.5, 50, 1500),
                    0.05, 0.35, 0.02, 3.0, seed, prefix=b"prot")


def dna_families(n_seqs=200_000, n_families=20_000, seed=2) -> SeqSet:
    return families(n_seqs, n_families, NUCLEO, NUCLEO_FREQ, _uniform_roots(200, 3000),
                    0.01, 0.10, 0.01, 2.0, seed, prefix=b"dna")


def _family_chunk(args):
    """Worker of families_parallel: one chunk of families from its own seed."""
    (seed, f0, f1, per, alphabet, freqs, root_len_fn, sub_lo, sub_hi, indel_rate, indel_mean,
     prefix) = args
    rng = np.random.default_rng(seed)
    rl = root_len_fn(rng, f1 - f0).astype(np.int64)
    roots = _draw(rng, alphabet, freqs, int(rl.sum()))
    out, lens, fam = _mutate_chunk(rng, roots, rl, per, alphabet, freqs, sub_lo, sub_hi,
                                   indel_rate, indel_mean)
    if prefix is None:  # no names (large sets that never become FASTA)
        return out, lens, None
    mem = np.concatenate([np.arange(k) for k in per])
    names = [b">%s%07d_%02d" % (prefix, f0 + fam[i], mem[i]) for i in range(len(fam))]
    return out, lens, names


def families_parallel(n_seqs, n_families, alphabet, freqs, root_len_fn, sub_lo, sub_hi,
                      indel_rate, indel_mean, seed, chunk_families=5000, prefix=b"fam",
                      workers=0) -> SeqSet:
    """families() for large sets: every chunk of families draws from its own
    child seed (numpy SeedSequence), so chunks are generated in parallel
    processes (spawned) and the result does not depend on the worker count.
    Sequences are in generation order (family-major)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import os
    per = np.full(n_families, n_seqs // n_families, dtype=np.int64)
    per[: n_seqs - int(per.sum())] += 1
    starts = list(range(0, n_families, chunk_families))
    seeds = np.random.SeedSequence(seed).spawn(len(starts))
    jobs = [(seeds[k], f0, min(n_families, f0 + chunk_families),
             per[f0:min(n_families, f0 + chunk_families)], alphabet, freqs, root_len_fn,
             sub_lo, sub_hi, indel_rate, indel_mean, prefix) for k, f0 in enumerate(starts)]
    workers = workers or min(len(jobs), os.cpu_count() or 1)
    if workers > 1:
        with cf.ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
            parts = list(ex.map(_family_chunk, jobs))
    else:
        parts = [_family_chunk(j) for j in jobs]
    residues = np.concatenate([p[0] for p in parts])
    lens = np.concatenate([p[1] for p in parts])
    names = [nm for p in parts for nm in p[2]] if prefix is not None else []
    return SeqSet(residues, lens, names)


def packed_proteins(n_seqs, n_families, seed=5):
    """A large protein database as packed records, without FASTA: the
    small-protein generator (log-normal roots median 300, sigma 0.5, 50-1500;
    5-35 % substitutions, 2 % indels of mean 3), index order = length
    descending (stable), packed on the device.  Returns (packed words, word
    offsets, lengths)."""
    from . import pack_records
    fam = families_parallel(n_seqs, n_families, AMINO, AMINO_FREQ,
                            _lognormal_roots(300, 0.5, 50, 1500), 0.05, 0.35, 0.02, 3.0, seed,
                            prefix=None)
    order = np.argsort(-fam.lens, kind="stable")
    lens = fam.lens[order].astype(np.uint32)
    packed, offs = pack_records(fam.residues, fam.starts[order].astype(np.uint64), lens)
    return packed, offs, lens


def serving_set(n_db=2_000_000, n_queries=300_000, n_families=100_000, novel=0.1, seed=4,
                subs=(0.05, 0.35), indels=(0.02, 3.0)):
    """The serving workload: sequences of the small-protein generator (log-normal
    roots, median 300, sigma 0.5, 50-1500; by default 5-35 % substitutions, 2 %
    indels of mean 3) from n_families families, split at random into a
    database of n_db (index order: length descending) and held-out queries; a
    share `novel` of the queries are unrelated sequences (new clusters).
    subs=(0, 0.04), indels=(0.005, 2) gives close relatives, most of which
    reach identity 90 against their family.  Returns (database SeqSet,
    queries SeqSet in random order)."""
    n_rel = int(round(n_queries * (1 - novel)))
    fam = families_parallel(n_db + n_rel, n_families, AMINO, AMINO_FREQ,
                            _lognormal_roots(300, 0.5, 50, 1500), subs[0], subs[1], indels[0],
                            indels[1], seed, prefix=b"srv")
    rng = np.random.default_rng(seed + 1)
    perm = rng.permutation(len(fam))
    db_ids, q_ids = perm[:n_db], perm[n_db:]
    db_ids = db_ids[np.argsort(-fam.lens[db_ids], kind="stable")]

    def subset(ids):
        idx = _gather_runs(fam.starts[ids], fam.lens[ids])
        return fam.residues[idx], fam.lens[ids], [fam.names[i] for i in ids]

    db = SeqSet(*subset(db_ids))
    qr, ql, qn = subset(q_ids)
    n_nov = n_queries - n_rel
    nl = _lognormal_roots(300, 0.5, 50, 1500)(rng, n_nov).astype(np.int64)
    nov = _draw(rng, AMINO, AMINO_FREQ, int(nl.sum()))
    res = np.concatenate([qr, nov])
    lens = np.concatenate([ql, nl])
    names = qn + [b">novel%07d" % k for k in range(n_nov)]
    order = rng.permutation(len(lens))
    starts = np.concatenate([[0], np.cumsum(lens)[:-1]])
    q = SeqSet(res[_gather_runs(starts[order], lens[order])], lens[order],
               [names[i] for i in order])
    return db, q


def _heavy_tailed_roots(rng, k):
    """80 % log-normal (median 250, sigma 0.5, at least 10), 19 % uniform
    1,000-5,000, 1 % uniform 5,000-35,000."""
    u = rng.random(k)
    out = np.clip(np.round(rng.lognormal(np.log(250), 0.5, size=k)), 10, 5000)
    mid = (u >= 0.80) & (u < 0.99)
    out[mid] = rng.integers(1000, 5001, size=int(mid.sum()))
    top = u >= 0.99
    out[top] = rng.integers(5000, 35001, size=int(top.sum()))
    return out


class PairSet:
    """A database in index order (length descending, as makedb orders it) and
    candidate pairs (rep, tar) of indices with rep < tar."""

    def __init__(self, seqs: SeqSet, pairs: np.ndarray, related: np.ndarray):
        self.seqs = seqs
        self.pairs = pairs
        self.related = related


def protein_pairs(n_pairs=2_000_000, seed=3, family_size=5, window=64) -> PairSet:
    """Heavy-tailed protein candidate pairs: half are pairs within one family
    (the root and members at 50-99 % identity to it: 1-50 % substitutions,
    1 % indels of mean length 2; every pair of the family's sequences), half
    pair unrelated sequences of similar length (a random partner within
    `window` places in length order, from another family)."""
    rng = np.random.default_rng(seed)
    per_family = family_size * (family_size - 1) // 2
    n_fam = max(1, (n_pairs // 2 + per_family - 1) // per_family)
    fams = families(n_fam * family_size, n_fam, AMINO, AMINO_FREQ, _heavy_tailed_roots,
                    0.01, 0.50, 0.01, 2.0, seed, prefix=b"pair", with_root=True)
    fam_of = np.array([int(nm[5:].split(b"_")[0]) for nm in fams.names], dtype=np.int64)
    # index order: length descending, stable in generation order
    order = np.argsort(-fams.lens, kind="stable")
    idx = _gather_runs(fams.starts[order], fams.lens[order])
    seqs = SeqSet(fams.residues[idx], fams.lens[order], [fams.names[i] for i in order])
    fam = fam_of[order]
    # related pairs: every pair of members of a family
    by_fam = np.argsort(fam, kind="stable")
    members = by_fam.reshape(n_fam, family_size)
    a, b = np.triu_indices(family_size, 1)
    rel = np.stack([members[:, a].reshape(-1), members[:, b].reshape(-1)], axis=1)
    rel = rel[: n_pairs // 2]
    # unrelated pairs: neighbours in length order from other families
    n_un = n_pairs - len(rel)
    i = rng.integers(0, len(seqs), size=n_un)
    j = np.clip(i + rng.integers(1, window + 1, size=n_un) * rng.choice([-1, 1], size=n_un),
                0, len(seqs) - 1)
    ok = (fam[i] != fam[j]) & (i != j)
    while not ok.all():  # redraw inside the window around i
        bad = np.flatnonzero(~ok)
        lo = np.maximum(i[bad] - window, 0)
        hi = np.minimum(i[bad] + window, len(seqs) - 1)
        j[bad] = lo + (rng.random(len(bad)) * (hi - lo + 1)).astype(np.int64)
        ok = (fam[i] != fam[j]) & (i != j)
    un = np.stack([i, j], axis=1)
    pairs = np.concatenate([rel, un])
    pairs.sort(axis=1)  # rep = the lower index = the longer record
    related = np.concatenate([np.ones(len(rel), bool), np.zeros(n_un, bool)])
    perm = rng.permutation(len(pairs))
    return PairSet(seqs, pairs[perm].astype(np.uint32), related[perm])
