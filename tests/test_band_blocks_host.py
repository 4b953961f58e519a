"""The library's count of the 32x32 blocks a pair's band visits
(common.cuh band_blocks: a closed form of the reference loop, used for the
reported aligned cells) against the oracle's loop (ngo_band_blocks), for
every identity, both rounding forms and a grid of lengths.  The library's
header is compiled on the host with nvcc together with the oracle's C
restatement; no GPU."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r'''
#include <cstdio>
#include <cstdint>
#include "common.cuh"
extern "C" {
#include "ngia_oracle.h"
}
int main() {
  long checked = 0, bad = 0;
  for (uint32_t id = 1; id <= 99; ++id) {
    for (int mode = 0; mode < 2; ++mode) {
      const float t = ngia::identity_threshold(id);
      for (uint32_t lr = 1; lr <= 9000; lr += lr < 300 ? 1 : 97) {
        for (uint32_t lt = 1; lt <= 9000; lt += lt < 300 ? 3 : 89) {
          const uint64_t got = ngia::band_blocks(ngia::make_band(lr, lt, t, mode));
          const uint64_t want = ngo_band_blocks(lr, lt, id, mode);
          ++checked;
          if (got != want && bad++ < 5)
            printf("id %u mode %d lr %u lt %u got %llu want %llu\n", id, mode, lr, lt,
                   (unsigned long long)got, (unsigned long long)want);
        }
      }
    }
  }
  printf("checked %ld bad %ld\n", checked, bad);
  return bad != 0;
}
'''


def test_closed_form_band_blocks_equal_the_loop(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    src = tmp_path / "bb.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "bb"
    build = subprocess.run(
        [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
         "-I", str(ROOT / "ngia2_gb300" / "csrc"), "-I", str(ROOT / "include"),
         "-I", str(ROOT / "oracle"), str(src), str(ROOT / "oracle" / "ngia_oracle.c"),
         "-o", str(exe)], capture_output=True, text=True, timeout=300)
    assert build.returncode == 0, build.stderr[-2000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout[-2000:]
    assert "bad 0" in run.stdout
