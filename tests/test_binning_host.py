"""The batched aligner's binning (align.cuh width_class) compiled on the host
with nvcc and checked over a grid of lengths, every identity, both band
roundings and several plans: each pair lands in a class that can hold it --
a streaming class at least as wide as its window (the narrowest such), a
group class whose lanes hold one live slice each, the general kernel only
when nothing narrower takes it, the skip class exactly when the length filter
fails -- and its queue key leads with its class.  The default plan's classes
also equal the Python mirror the GPU tests use.  No GPU."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r'''
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include "align.cuh"
using namespace ngia;

static long checked = 0, bad = 0;
#define CHECK(cond, ...) do { ++checked; if (!(cond) && bad++ < 8) { \
  printf("FAIL %s: ", #cond); printf(__VA_ARGS__); printf("\n"); } } while (0)

static void check(const Band &b, const ClassPlan &p, uint32_t id, int mode) {
  const int c = width_class(b, p);
  const uint32_t ws = stream_width(b);
  const char *fmt = "lr %u lt %u id %u mode %d class %d ws %u stream_max %u";
#define ARGS b.lr, b.lt, id, mode, c, ws, p.stream_max
  CHECK((c == kSkipClass) == !b.pass, fmt, ARGS);
  CHECK(c >= 0 && c < kNumClasses, fmt, ARGS);
  CHECK((class_sort_key(c, b) >> 3) == (uint32_t)c, fmt, ARGS);
  if (c < kNumLdsClasses) {
    CHECK(ws <= p.stream_max && (uint32_t)class_width(c) >= ws, fmt, ARGS);
    CHECK(c == 0 || (uint32_t)class_width(c - 1) < ws, fmt, ARGS);
  } else if (c < kGeneralClass) {
    const int g = c - kFirstGroupClass;
    const GroupShape sh = group_shape(c);
    const uint32_t ns = (b.nr + sh.K - 1) / sh.K;
    CHECK(ws > p.stream_max && p.group_limit[g] != 0, fmt, ARGS);
    CHECK(ns <= (uint32_t)sh.G || b.ls + b.rs <= p.group_limit[g], fmt, ARGS);
    CHECK(group_fits(b, sh.G, sh.K), fmt, ARGS);
    for (int h = 0; h < g; ++h) {  // no earlier group class takes it
      const GroupShape s2 = group_shape(kFirstGroupClass + h);
      const uint32_t n2 = (b.nr + s2.K - 1) / s2.K;
      CHECK(p.group_limit[h] == 0 || !(n2 <= (uint32_t)s2.G || b.ls + b.rs <= p.group_limit[h]),
            fmt, ARGS);
    }
  } else if (c == kGeneralClass) {
    CHECK(ws > p.stream_max && b.nr <= 2048, fmt, ARGS);
    for (int h = 0; h < kNumGroupClasses; ++h) {
      const GroupShape s2 = group_shape(kFirstGroupClass + h);
      const uint32_t n2 = (b.nr + s2.K - 1) / s2.K;
      CHECK(p.group_limit[h] == 0 || !(n2 <= (uint32_t)s2.G || b.ls + b.rs <= p.group_limit[h]),
            fmt, ARGS);
    }
  }
#undef ARGS
}

int main(int argc, char **argv) {
  ClassPlan plans[6];
  plans[0] = default_plan();
  plans[1] = default_plan(); plans[1].stream_max = 4;
  plans[2] = default_plan(); plans[2].stream_max = 8;
  plans[3] = default_plan(); plans[3].stream_max = 12;
  for (int g = 0; g < kNumGroupClasses; ++g) plans[3].group_limit[g] = 0;
  plans[4] = default_plan(); plans[4].stream_max = 4;
  plans[4].group_limit[0] = plans[4].group_limit[2] = plans[4].group_limit[4] = 0;
  plans[5] = default_plan(); plans[5].stream_max = 16;
  plans[5].group_limit[0] = 20; plans[5].group_limit[3] = 100; plans[5].group_limit[5] = 0;
  uint32_t lens[400];
  int nl = 0;
  for (uint32_t L = 1; L <= NGIA_MAX_READ + 2 && nl < 400; L += L < 64 ? 3 : L < 2048 ? L / 9 : L / 5)
    lens[nl++] = L;
  lens[nl++] = NGIA_MAX_READ;
  for (uint32_t id = 1; id <= 99; ++id)
    for (int mode = 0; mode < 2; ++mode)
      for (int a = 0; a < nl; ++a)
        for (int c = 0; c < nl; ++c) {
          const Band b = make_band(lens[a], lens[c], identity_threshold(id), mode);
          for (const ClassPlan &p : plans) check(b, p, id, mode);
        }
  // the default plan's classes for the Python mirror
  if (argc > 1) {
    FILE *f = fopen(argv[1], "w");
    for (uint32_t id = 30; id <= 95; id += 5)
      for (int a = 0; a < nl; a += 3)
        for (int c = 0; c < nl; c += 3)
          fprintf(f, "%u %u %u %d\n", lens[a], lens[c], id,
                  width_class(make_band(lens[a], lens[c], identity_threshold(id), 1)));
    fclose(f);
  }
  printf("checked %ld bad %ld\n", checked, bad);
  return bad != 0;
}
'''


def test_every_pair_lands_in_a_class_that_holds_it(tmp_path, built):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    src = tmp_path / "bins.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "bins"
    build = subprocess.run(
        [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-I", str(ROOT / "ngia2_gb300" / "csrc"),
         "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
        capture_output=True, text=True, timeout=600)
    assert build.returncode == 0, build.stderr[-2000:]
    table = tmp_path / "classes.txt"
    run = subprocess.run([str(exe), str(table)], capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stdout[-2000:]
    assert "bad 0" in run.stdout

    from test_gpu_batched import width_class
    rows = [tuple(int(x) for x in line.split()) for line in table.read_text().splitlines()]
    assert len(rows) > 1000
    seen = set()
    for lr, lt, identity, cls in rows:
        assert width_class(lr, lt, identity) == cls, (lr, lt, identity, cls)
        seen.add(cls)
    import ngia2_gb300 as ng
    assert {0, 10, ng.GENERAL_CLASS, ng.SKIP_CLASS} <= seen, sorted(seen)
    assert set(range(ng.FIRST_GROUP_CLASS, ng.GENERAL_CLASS)) & seen, sorted(seen)
