"""Host arithmetic of the evaluator's work layout (no GPU), checked by host
programs compiled against the kernels' own header.

DP tiles: `dp_tile_groups` gives the number of
L-record groups per tile of T slots.  The whole-quad kernels read direct
columns as aligned 16-byte quads and stage tiles with bulk copies, which
is safe only where every tile starts on a multiple of 4 records; the tile
must hold whole groups (each group is reduced by its own tree, then the
groups are added in record order), fit the T slots, and be as large as
those rules allow.  Checked for every lane count at the three tile sizes
the evaluator uses.

Chunked work items: `chunk_item` maps the chunked kernels' queue index to
(record chunk, program), the programs in groups and each group
chunk-major.  Every pair must be exactly one item, and a program's previous
chunk must have a smaller index (the bounded wait is then always on an item
an earlier CTA holds)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DP_SRC = r"""
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


CHUNK_SRC = r"""
#include <cstdio>
#include <vector>
#include "ppi_internal.cuh"
int main() {
   int bad = 0, cases = 0;
   for (int limit : {1, 2, 7, 100, 2048, 5000})
      for (int group : {1, 3, 64, 2048, 4700, 1 << 30})
         for (int nc : {1, 2, 5, 62}) {
            ++cases;
            std::vector<long long> at((size_t)limit * nc, -1);
            const long long items = (long long)limit * nc;
            for (long long it = 0; it < items; ++it) {
               int c = -1, k = -1;
               ppi::chunk_item(it, limit, group, nc, &c, &k);
               if (c < 0 || c >= nc || k < 0 || k >= limit) { ++bad; break; }
               long long& slot = at[(size_t)k * nc + c];
               if (slot >= 0) { ++bad; break; }   // two items on one pair
               slot = it;
            }
            for (int k = 0; k < limit && !bad; ++k)
               for (int c = 1; c < nc; ++c)
                  if (at[(size_t)k * nc + c] <= at[(size_t)k * nc + c - 1]) { ++bad; break; }
            if (bad) {
               std::printf("limit=%d group=%d chunks=%d\n", limit, group, nc);
               return 1;
            }
         }
   std::printf("cases=%d bad=%d\n", cases, bad);
   return 0;
}
"""


def _run(tmp_path, name, source):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / (name + ".cu")
    src.write_text(source)
    exe = str(tmp_path / name)
    subprocess.run([nvcc, "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "ppi-auto_gb300", "csrc"), str(src), "-o", exe],
                   check=True, capture_output=True, text=True)
    return subprocess.run([exe], capture_output=True, text=True)


def test_chunk_items_cover_every_pair_once_in_chunk_order(tmp_path):
    r = _run(tmp_path, "chunk_items", CHUNK_SRC)
    assert r.returncode == 0, r.stdout
    assert "cases=144 bad=0" in r.stdout


def test_dp_tile_groups_whole_quads(tmp_path):
    r = _run(tmp_path, "dp_tiles", DP_SRC)
    assert r.returncode == 0, r.stdout
    # every lane count up to a quarter of the tile, and every multiple of 4,
    # tiles in whole quads
    checked, aligned = (int(x.split("=")[1]) for x in r.stdout.split()[-3:-1])
    assert checked == 256 + 512 + 1024
    assert aligned >= sum(T // 4 + (T - T // 4) // 4 for T in (256, 512, 1024))
