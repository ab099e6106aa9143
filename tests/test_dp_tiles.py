"""DP tiles (host arithmetic, no GPU): `dp_tile_groups` gives the number of
L-record groups per tile of T slots.  The whole-quad kernels read direct
columns as aligned 16-byte quads and stage tiles with bulk copies, which
is safe only where every tile starts on a multiple of 4 records; the tile
must hold whole groups (each group is reduced by its own tree, then the
groups are added in record order), fit the T slots, and be as large as
those rules allow.  Checked for every lane count at the three tile sizes
the evaluator uses, by a host program compiled against the kernels' own
header."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <cstdio>
#include "ppi_internal.cuh"
int main() {
   int bad = 0, aligned = 0, total = 0;
   for (int T : {256, 512, 1024})
      for (int L = 1; L <= T; ++L) {
         const int g = ppi::dp_tile_groups(L, T);
         int best = 0;   // the most whole groups that make a whole-quad tile
         for (int k = 1; k * L <= T; ++k)
            if ((k * L) % 4 == 0) best = k;
         const int want = best > 0 ? best : T / L;
         ++total;
         if ((g * L) % 4 == 0) ++aligned;
         if (g != want || g < 1 || g * L > T) {
            ++bad;
            std::printf("T=%d L=%d groups=%d want=%d\n", T, L, g, want);
         }
      }
   std::printf("checked=%d aligned=%d bad=%d\n", total, aligned, bad);
   return bad != 0;
}
"""


def test_dp_tile_groups_whole_quads(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "dp_tiles.cu"
    src.write_text(SRC)
    exe = str(tmp_path / "dp_tiles")
    subprocess.run([nvcc, "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "ppi-auto_gb300", "csrc"), str(src), "-o", exe],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    # every lane count up to a quarter of the tile, and every multiple of 4,
    # tiles in whole quads
    checked, aligned = (int(x.split("=")[1]) for x in r.stdout.split()[-3:-1])
    assert checked == 256 + 512 + 1024
    assert aligned >= sum(T // 4 + (T - T // 4) // 4 for T in (256, 512, 1024))
