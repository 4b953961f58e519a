"""Times the reference's own GPU build against ngia2 on one workload and
checks that both write the same result file.  TEST INFRASTRUCTURE ONLY.

Runs, on the same GPU and the same input:
  oracle/_ref/ngia2_gpu -m makedb / -m clustering / -m fast   (the reference,
      built unmodified by nvcc; makedb runs on the host with OpenMP)
  ngia2_gb300/lib/ngia2  -m makedb / -m clustering / -m fast   (this library)
and prints one JSON object with wall times, the reference's own stage timers
and whether the packed files and result files are byte-identical.

    python oracle/time_reference_gpu.py [--n-seqs 200000] [--identity 95] [--out f.json]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import re
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def sha(p: Path) -> str:
    return hashlib.sha256(p.read_bytes()).hexdigest()


LOGS: list = []


def run(cmd, timeout=3600):
    t0 = time.perf_counter()
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True, timeout=timeout)
    dt = time.perf_counter() - t0
    LOGS.append((" ".join(str(c) for c in cmd), r.stdout))
    if r.returncode != 0:
        raise RuntimeError(f"{cmd[0]} failed ({r.returncode}):\n{r.stdout[-2000:]}{r.stderr[-2000:]}")
    return dt, r.stdout


def consuming(out: str, tag: str):
    """Seconds of the reference's Timer line that follows `tag`."""
    m = re.search(re.escape(tag) + r"\s*Consuming:\s*(\d+) h\s*(\d+) m\s*(\d+) s\s*(\d+) ms\s*(\d+) us",
                  out)
    if not m:
        return None
    h, mi, s, ms, us = map(int, m.groups())
    return h * 3600 + mi * 60 + s + ms / 1e3 + us / 1e6


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kind", choices=["dna", "protein"], default="dna")
    ap.add_argument("--n-seqs", type=int, default=200_000)
    ap.add_argument("--families", type=int, default=0)
    ap.add_argument("--identity", type=int, default=95)
    ap.add_argument("--bands", type=int, default=64)
    ap.add_argument("--out", default="")
    ap.add_argument("--log-dir", default="", help="keep every command's stdout here")
    a = ap.parse_args()
    import ngia2_gb300 as ng
    from ngia2_gb300 import synth
    import oracle
    ref = oracle.ref_gpu_cli()
    if not ref.exists():
        raise SystemExit("reference GPU build missing: run oracle/build.sh")
    fam = a.families or max(1, a.n_seqs // 10)
    d = Path(tempfile.mkdtemp(prefix="ngia_refgpu_"))
    if a.kind == "dna":
        s = synth.dna_families(a.n_seqs, fam, 2)
    else:
        s = synth.protein_families(a.n_seqs, fam, 1)
    fa = d / "w.fa"
    s.write_fasta(fa)
    res = {"workload": f"{a.n_seqs} {a.kind} sequences, {fam} families, identity {a.identity}, "
                       f"{a.bands} bands", "gpu": "same GPU, one process at a time"}
    t, out = run([ref, "-m", "makedb", "-f", fa, "-p", d / "ref.packed"])
    res["ref_makedb_s"] = t
    t, out = run([ng.CLI_PATH, "-m", "makedb", "-f", fa, "-p", d / "ours.packed"])
    res["ours_makedb_s"] = t
    res["packed_identical"] = sha(d / "ref.packed") == sha(d / "ours.packed")
    for mode in ("clustering", "fast"):
        args = ["-m", mode, "-p", d / "ref.packed", "-r", d / f"ref_{mode}.txt",
                "-i", str(a.identity), "-b", str(a.bands)]
        t, out = run([ref, *args])
        res[f"ref_{mode}_s"] = t
        if mode == "clustering":
            res["ref_align_s"] = consuming(out, f"[align {a.bands} bands]")
            res["ref_buildgraph_sort_s"] = consuming(out, "[buildGraph]")
            m = re.search(r"compare pairs:\s*(\d+)", out)
            res["ref_compare_pairs"] = int(m.group(1)) if m else None
        args[5] = d / f"ours_{mode}.txt"
        t, out = run([ng.CLI_PATH, *args])
        res[f"ours_{mode}_s"] = t
        m = re.search(r"\[%s\]\s*([0-9.]+) s" % mode if mode == "fast" else r"\[clustering\]\s*([0-9.]+) s", out)
        res[f"ours_{mode}_inner_s"] = float(m.group(1)) if m else None
        res[f"{mode}_result_identical"] = sha(d / f"ref_{mode}.txt") == sha(d / f"ours_{mode}.txt")
    line = json.dumps(res)
    print(line)
    if a.log_dir:
        Path(a.log_dir).mkdir(parents=True, exist_ok=True)
        for k, (cmd, out) in enumerate(LOGS):
            (Path(a.log_dir) / f"run{k:02d}.txt").write_text(cmd + "\n\n" + out)
    if a.out:
        Path(a.out).write_text(line + "\n")


if __name__ == "__main__":
    main()
