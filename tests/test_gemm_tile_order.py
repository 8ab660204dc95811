"""Host check of the tcgen05 GEMM's tile order (csrc/gemm_tiles.cuh).

The kernel maps its block index to a (row tile, column tile) pair with
``tile_of`` and the host launches ``tile_count`` blocks.  Every valid tile
must be produced exactly once: all tm x tn tiles for the column-sum GEMM,
the tiles with tm < 2 tn + 2 for the symmetric (upper-triangle) Gram.  The
header is plain C++ without nvcc, so it is compiled here with the host
compiler and checked exhaustively over a range of shapes, including the
64-site step's (33,280 rows: 260 x 130 tiles; SNR 128 x 130 tiles).
"""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "vmc_jax_gb300", "csrc")

CHECK = r"""
#include "gemm_tiles.cuh"
#include <cstdio>
#include <vector>
using namespace vmc;

static long check(int mode, int tM, int tN) {
  const int64_t n = tile_count(mode, tM, tN);
  std::vector<char> seen((size_t)tM * tN, 0);
  long bad = 0;
  for (int64_t b = 0; b < n; ++b) {
    int tm = -1, tn = -1;
    tile_of((int)b, mode, tM, tN, tm, tn);
    if (tm < 0 || tm >= tM || tn < 0 || tn >= tN || (mode == 0 && tm >= 2 * tn + 2) ||
        seen[(size_t)tm * tN + tn]) {
      ++bad;
      continue;
    }
    seen[(size_t)tm * tN + tn] = 1;
  }
  int64_t valid = 0;
  for (int tm = 0; tm < tM; ++tm)
    for (int tn = 0; tn < tN; ++tn)
      if (mode != 0 || tm < 2 * tn + 2) valid += seen[(size_t)tm * tN + tn] ? 1 : 0;
  int64_t want = 0;
  for (int tm = 0; tm < tM; ++tm)
    for (int tn = 0; tn < tN; ++tn) want += (mode != 0 || tm < 2 * tn + 2) ? 1 : 0;
  if (valid != want || n != want) ++bad;
  return bad;
}

int main() {
  long bad = 0, cases = 0;
  for (int rows = 1; rows <= 40000; rows += rows < 3000 ? 37 : 997) {  // square Gram
    bad += check(0, (rows + 127) / 128, (rows + 255) / 256);
    ++cases;
  }
  for (int tM = 1; tM <= 140; tM += tM < 20 ? 1 : 9)  // column sums of an m x n product
    for (int tN = 1; tN <= 140; tN += tN < 20 ? 1 : 11) {
      bad += check(1, tM, tN);
      ++cases;
    }
  bad += check(0, 260, 130) + check(1, 128, 130) + check(0, 64, 32) + check(1, 128, 32);
  printf("%ld %ld\n", cases + 4, bad);
  return bad != 0;
}
"""


def test_tile_order_is_a_bijection(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "tile_order_check.cpp"
    exe = tmp_path / "tile_order_check"
    src.write_text(CHECK)
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    cases, bad = map(int, r.stdout.split())
    assert bad == 0 and cases > 100
