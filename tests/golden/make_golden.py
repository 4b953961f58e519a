"""Generates the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own makedb, alignment kernel, buildGraph, Leiden, fast
clustering and SaveResult code, built as a host (OpenMP) program by
oracle/build.sh, on small seeded inputs, and stores inputs and outputs:

  <name>.fa.gz                   FASTA input (multi-line records, edge cases)
  <name>.packed.gz               reference makedb output (rep rows grouped)
  <name>.sigs.npy                reference signatures, seq-major [n][64]
                                 (makedb without the grouping step)
  <name>.pairs_<id>.npz          every distinct candidate pair of 64 bands with
                                 the reference kernel's score, both band-bound
                                 roundings (score_split, score_fma)
  <name>.edges_<id>_<mode>.npy   reference buildGraph edge list (rep, tar, score)
  <name>.leiden_<id>.npy         reference Leiden clusters on those edges
  <name>.fast_<id>.npy           reference fast-mode clusters
  <name>.result_<id>.sha256      sha256 of the reference result file
  known_answer.npz               hand-checkable LCS cases (see below)

Run from the repository root on a machine with the reference checkout:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import gzip
import hashlib
import shutil
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from ngia2_gb300 import synth  # noqa: E402
import ngia2_gb300 as ng  # noqa: E402

GOLDEN = Path(__file__).resolve().parent
IDENTITIES = {"prot": (50, 70, 90), "dna": (80, 90, 95), "edge": (30, 50, 90)}


def edge_case_set() -> synth.SeqSet:
    """Sequences exercising the format's corners."""
    rng = np.random.default_rng(11)
    seqs: list[bytes] = []
    names: list[bytes] = []

    def add(name: bytes, s: bytes):
        names.append(name)
        seqs.append(s)

    base = synth._draw(rng, synth.AMINO, synth.AMINO_FREQ, 4000).tobytes()
    add(b">long_root", base)
    for k in range(3):  # long relatives: wide bands at low identity
        s = bytearray(base)
        for p in rng.choice(len(s), size=400 + 200 * k, replace=False):
            s[p] = synth.AMINO[rng.integers(0, 20)]
        add(b">long_rel%d" % k, bytes(s[: len(s) - 150 * k]))
    add(b">lower_case", base[:300].lower())
    add(b">mixed_case", base[:300:2] + base[300:600:2].lower())
    add(b">unknown_letters", b"XBZJOU*-.0123" + base[:200] + b"XXXX")
    for L in (1, 2, 5, 7, 8, 9, 31, 32, 33, 63, 64, 65):
        add(b">short_%d" % L, base[1000:1000 + L])
        add(b">short_%d_copy" % L, base[1000:1000 + L])
    add(b">empty_a", b"")
    add(b">empty_b", b"")
    add(b">dna_n", b"ACGTNNNNACGTUUACGT" * 20)
    add(b">dna_n_copy", b"ACGTNNNNACGTUUACGT" * 20)
    add(b">too_long_dropped", b"A" * 0xFFFF)
    add(b">just_fits", (b"ACDEFGHIKL" * 6554)[:0xFFFE])
    add(b">just_fits_copy", (b"ACDEFGHIKL" * 6554)[:0xFFFE])
    fam = synth.protein_families(120, 12, seed=13)
    for i in range(len(fam)):
        add(fam.names[i], fam.seq(i))
    order = rng.permutation(len(seqs))
    lens = np.array([len(seqs[i]) for i in order])
    res = np.frombuffer(b"".join(seqs[i] for i in order), np.uint8)
    return synth.SeqSet(res.copy(), lens, [names[i] for i in order])


def sets():
    return {
        "prot": (synth.protein_families(600, 60, seed=21), 60),
        "dna": (synth.dna_families(400, 40, seed=22), 0),
        "edge": (edge_case_set(), 70),
    }


def sha(path: Path) -> str:
    return hashlib.sha256(path.read_bytes()).hexdigest()


def main() -> None:
    oracle.build()
    tmp = Path(tempfile.mkdtemp())
    for name, (seqset, width) in sets().items():
        fa = tmp / f"{name}.fa"
        seqset.write_fasta(fa, line_width=width)
        packed = tmp / f"{name}.packed"
        nog = tmp / f"{name}.nogroup.packed"
        assert oracle.ref_makedb(fa, nog, group=False) == 0
        assert oracle.ref_makedb(fa, packed) == 0
        with gzip.open(GOLDEN / f"{name}.fa.gz", "wb", compresslevel=9) as f:
            f.write(fa.read_bytes())
        with gzip.open(GOLDEN / f"{name}.packed.gz", "wb", compresslevel=9) as f:
            f.write(packed.read_bytes())
        db = ng.read_packed(packed)
        n = db["n"]
        raw = ng.read_packed(nog)["raw"]
        sigs = raw[4 + 24 * n: 4 + 24 * n + 256 * n].view(np.uint32).reshape(n, 64)
        np.save(GOLDEN / f"{name}.sigs.npy", sigs)
        for ident in IDENTITIES[name]:
            cand = np.concatenate([oracle.collect_band(db["rep"][b], db["lens"], ident)
                                   for b in range(64)])
            uniq = np.unique(cand, axis=0) if len(cand) else np.zeros((0, 2), np.uint32)
            s_split = oracle.ref_align_jobs(db["packed"], db["offsets"], uniq, ident,
                                            oracle.ROUND_SPLIT)
            s_fma = oracle.ref_align_jobs(db["packed"], db["offsets"], uniq, ident,
                                          oracle.ROUND_FMA)
            np.savez_compressed(GOLDEN / f"{name}.pairs_{ident}.npz", pairs=uniq,
                                score_split=s_split, score_fma=s_fma,
                                candidates=np.uint64(len(cand)))
            for mode, tag in ((oracle.ROUND_SPLIT, "split"), (oracle.ROUND_FMA, "fma")):
                r, t, w = oracle.ref_build_graph(packed, ident, 64, 1 << 20, mode)
                sc = np.rint(w.astype(np.float64) * 100).astype(np.int64)
                np.save(GOLDEN / f"{name}.edges_{ident}_{tag}.npy",
                        np.stack([r, t, sc], axis=1).astype(np.int64))
            r, t, w = oracle.ref_build_graph(packed, ident, 64, 1 << 20, oracle.ROUND_FMA)
            clu = oracle.ref_leiden(r, t, w, n, ng_resolution(ident))
            np.save(GOLDEN / f"{name}.leiden_{ident}.npy", clu)
            fast = oracle.ref_fast_cluster(packed, ident, 64, n, oracle.ROUND_FMA)
            np.save(GOLDEN / f"{name}.fast_{ident}.npy", fast)
            res = tmp / f"{name}.result_{ident}.txt"
            oracle.ref_save(clu, packed, res)
            fres = tmp / f"{name}.fastresult_{ident}.txt"
            oracle.ref_save(fast, packed, fres)
            (GOLDEN / f"{name}.result_{ident}.sha256").write_text(
                f"{sha(res)}  leiden\n{sha(fres)}  fast\n")
    known_answers()
    shutil.rmtree(tmp)


def ng_resolution(identity: int) -> float:
    # (100 - |id - 50| * 2) / 100 in float32, clamped to [0, 1] (src/main.cu:114-116)
    r = np.float32((np.float32(100) - np.float32(abs(np.float32(identity) - np.float32(50)))
                    * np.float32(2)) / np.float32(100))
    return float(min(max(r, np.float32(0)), np.float32(1)))


def lcs_dp(a: bytes, b: bytes) -> int:
    """Textbook O(n*m) LCS over 4-bit codes; code 0 matches nothing."""
    ca = [oracle.residue_code(x) for x in a]
    cb = [oracle.residue_code(x) for x in b]
    prev = [0] * (len(cb) + 1)
    for i in range(1, len(ca) + 1):
        cur = [0] * (len(cb) + 1)
        for j in range(1, len(cb) + 1):
            if ca[i - 1] and ca[i - 1] == cb[j - 1]:
                cur[j] = prev[j - 1] + 1
            else:
                cur[j] = max(prev[j], cur[j - 1])
        prev = cur
    return prev[-1]


def known_answers() -> None:
    """Pairs whose band covers the whole matrix (rep <= 32 residues, low
    identity), so the banded LCS equals the textbook LCS; plus the identity
    score formula on hand-made cases."""
    rng = np.random.default_rng(31)
    reps, tars, lcs, ident = [], [], [], []
    for _ in range(300):
        lr = int(rng.integers(1, 33))
        lt = int(rng.integers(1, lr + 1))
        a = bytes(synth.AMINO[rng.integers(0, 4, size=lr)])
        b = bytes(synth.AMINO[rng.integers(0, 4, size=lt)])
        reps.append(a)
        tars.append(b)
        lcs.append(lcs_dp(a, b))
        ident.append(1)
    np.savez_compressed(GOLDEN / "known_answer.npz",
                        reps=np.frombuffer(b"".join(reps), np.uint8),
                        rep_lens=np.array([len(x) for x in reps]),
                        tars=np.frombuffer(b"".join(tars), np.uint8),
                        tar_lens=np.array([len(x) for x in tars]),
                        lcs=np.array(lcs), identity=np.array(ident))


if __name__ == "__main__":
    main()
