"""The placement of the register-tile Jacobi regions (span_count / span_own in
fluid_gb300/csrc/fg_internal.cuh), used by the per-launch kernel and by
batches: along an axis of n cells the regions' owned windows cover [0, n)
once, in order; a region edge inside the grid keeps a halo of 8 cells, one at
the grid's edge keeps none; column regions start on a multiple of 4 (16-byte
vector loads); and the count is the least any placement of 32-, 64- or
128-cell regions (4-warp rows, 8-warp rows, columns) with such halos needs.
The header's host side is compiled by nvcc into a small CPU program; no GPU
is used."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
#include <cstdio>
#include "fg_internal.cuh"
using namespace fg;

int main() {
  long long checked = 0;
  for (int R : {kJacRegionRows / 2, kJacRegionRows, kJacRegionCols}) {
    const int S = R - 2 * kJacHalo;
    for (int n = 1; n <= 5000; ++n) {
      const int cnt = span_count(n, R);
      const int least = n <= R ? 1 : (n - 2 * kJacHalo + S - 1) / S;
      if (cnt != least) { printf("count n=%d R=%d: %d, least %d\n", n, R, cnt, least); return 1; }
      int pos = 0;
      for (int t = 0; t < cnt; ++t) {
        const int a = t * S;
        const unsigned own = span_own(t, n, R);
        const int lo = own & 255, hi = own >> 8;
        const bool ok = a + lo == pos && lo < hi && hi <= R && (a == 0 || lo >= kJacHalo) &&
                        (a + R >= n || hi <= R - kJacHalo) && (R != kJacRegionCols || a % 4 == 0);
        if (!ok) { printf("region n=%d R=%d t=%d: a=%d own [%d, %d) pos %d\n", n, R, t, a, lo, hi, pos); return 1; }
        pos = a + hi;
        ++checked;
      }
      if (pos != n) { printf("cover n=%d R=%d: ends at %d\n", n, R, pos); return 1; }
    }
  }
  printf("ok %lld\n", checked);
  return 0;
}
"""


def test_region_placement_covers_each_axis_once_with_halos_inside_only(tmp_path):
    from fluid_gb300 import _build

    try:
        nvcc = _build.nvcc()
    except RuntimeError:
        pytest.skip("no CUDA toolkit")
    src = tmp_path / "regions.cu"
    exe = tmp_path / "regions"
    src.write_text(PROBE)
    subprocess.run([nvcc, "-std=c++17", "-I", os.path.join(ROOT, "fluid_gb300", "csrc"), "-I",
                    os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert out.stdout.startswith("ok ")
