"""Tile order of the mixed-precision 3D interior kernel (host-side check, no
GPU), for each of its tile heights: the launch enumerates every tile exactly
once, and the tiles it places first -- those that start without waiting for
the face kernels before them -- stage no face point and no ghost value
(their tile, 2-cell halo and the chunk's planes +-2 all lie in [1, n-2]).  Compiled with nvcc as host code
from the kernel's own header."""
import os
import shutil
import subprocess

import pytest

SRC = r'''
#include "kern_wide.cuh"
#include <cstdio>
#include <vector>
namespace nlse { namespace wide { int g_tile_order = 1; int g_pdl = 1; int g_face_bps = 8; int g_zc_override = 0; int g_z2 = 1; int g_wide_ty = 8; } }
using namespace nlse;
using namespace nlse::wide;
int check(int M, int N, int L, int zc, int cm, int TY) {
  Geom g; g.ndim = 3; g.M = M; g.N = N; g.L = L; g.n = (long long)M * N * L;
  const int TX = 32, H = 2;
  TileOrder t = tile_order(g, TX, TY, H, zc);
  t.chunk_major = cm;
  const long long nb = (long long)t.nbx * t.nby * t.nbz;
  std::vector<int> seen(nb, 0);
  for (long long b = 0; b < nb; ++b) {
    int bx, by, bz;
    t.tile((unsigned)b, bx, by, bz);
    if (bx < 0 || bx >= t.nbx || by < 0 || by >= t.nby || bz < 0 || bz >= t.nbz) return 1;
    seen[((long long)bz * t.nby + by) * t.nbx + bx]++;
    const int x0 = bx * TX, y0 = by * TY, z0 = bz * zc, z1 = z0 + zc < L ? z0 + zc : L;
    const bool inside = x0 - 2 >= 1 && x0 + TX + 1 <= M - 2 && y0 - H >= 1 &&
                        y0 + TY + H - 1 <= N - 2 && z0 - H >= 1 && z1 - 1 + H <= L - 2;
    if (!t.waits((unsigned)b) && !inside) return 2;  // a non-waiting tile touches a face
    if (t.waits((unsigned)b) && inside) return 3;    // an interior tile waits (allowed, but
                                                     // the order should not do it)
  }
  for (long long i = 0; i < nb; ++i)
    if (seen[i] != 1) return 4;
  return 0;
}
int main() {
  const int dims[] = {3, 4, 5, 9, 17, 31, 33, 34, 35, 36, 37, 40, 64, 65, 66, 67, 70, 97, 100, 129, 320};
  const int zcs[] = {1, 2, 3, 4, 5, 8, 16, 20, 33};
  long long n = 0;
  for (int M : dims) for (int N : dims) for (int L : {3, 4, 5, 8, 9, 20, 37, 64, 320})
    for (int zc : zcs) {
      if (zc > L) continue;
      for (int cm = 0; cm < 2; ++cm)
        for (int ty : {4, 8, 16}) {  // the tile heights of the interior kernel
          int r = check(M, N, L, zc, cm, ty);
          if (r) {
            printf("FAIL %d %d %d %d order %d ty %d code %d\n", M, N, L, zc, cm, ty, r);
            return 1;
          }
          ++n;
        }
    }
  printf("OK %lld\n", n);
  return 0;
}
'''


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
def test_tile_order_is_a_permutation_with_interior_first(tmp_path):
    from nlsemagic_gb300 import build as B
    src = tmp_path / "to.cu"
    src.write_text(SRC)
    exe = tmp_path / "to"
    cmd = [B.nvcc()] + B.ARCH + ["-O2", "-std=c++17", "--extended-lambda", "-I", B.CSRC,
                                 "-I", B.INCLUDE, str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith("OK"), out.stdout + out.stderr
