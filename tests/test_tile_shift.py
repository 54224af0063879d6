"""Tiling of the single-pass 2D and 1D stage kernels (host-side check, no
GPU), from the kernels' own headers: the shifted tiles (2D: 32 x TY for
every tile height; 1D: segments of 256 and 1024 points) cover every grid
point exactly once, no tile is empty, and no tile starts at 1 or n-1 --
so a boundary point shares its tile with its MSD neighbour, and an interior
point next to a face shares its tile with the face point whose ghost or D
it reads.  Compiled with nvcc as host code."""
import os
import shutil
import subprocess

import pytest

SRC = r'''
#include "kern_seg1d.cuh"
#include "kern_wide2d.cuh"
#include <cstdio>
namespace nlse { namespace wide { int g_pdl = 1; int g_wide2d = 1; int g_seg1d = 1; }
namespace wide2d { int g_ty = 0; } }
using namespace nlse;

// tiles of length t starting at t*b - s cover [0, n) once, none empty, none
// starting at 1 or n-1
static int check_axis(long long n, int t, int s, long long nb) {
  if (s != 0 && s != 1) return 1;
  if (t * nb - s < n) return 2;                     // coverage (the first tile starts at -s <= 0)
  if (t * (nb - 1) - s > n - 1) return 3;           // last tile not empty
  for (long long b = 0; b < nb; ++b) {
    const long long x0 = t * b - s;
    if (x0 == 1 || x0 == n - 1) return 4;
  }
  return 0;
}

int main() {
  long long cases = 0;
  for (int M = 3; M <= 200; ++M)
    for (int N : {3, 4, 5, 8, 9, 15, 16, 17, 31, 32, 33, 34, 63, 64, 65, 66, 97, 129, 130, 513}) {
      Geom g; g.ndim = 2; g.M = M; g.N = N; g.L = 1; g.n = (long long)M * N;
      for (int TY : {8, 16, 32}) {
        const int sx = wide2d::shift(M, wide2d::TX), sy = wide2d::shift(N, TY);
        const long long nbx = (M + sx + wide2d::TX - 1) / wide2d::TX;
        const long long nby = (N + sy + TY - 1) / TY;
        if (wide2d::tiles(g, TY) != nbx * nby) { printf("FAIL tiles %d %d %d\n", M, N, TY); return 1; }
        int r = check_axis(M, wide2d::TX, sx, nbx);
        if (!r) r = check_axis(N, TY, sy, nby);
        if (r) { printf("FAIL 2D %d %d %d code %d\n", M, N, TY, r); return 1; }
        ++cases;
      }
    }
  for (long long n = 3; n <= 5000; ++n) {
    int r = check_axis(n, 256, seg1d::shift<256>(n), seg1d::segments<256>(n));
    if (!r) r = check_axis(n, 1024, seg1d::shift<1024>(n), seg1d::segments<1024>(n));
    if (r) { printf("FAIL 1D %lld code %d\n", n, r); return 1; }
    ++cases;
  }
  printf("OK %lld\n", cases);
  return 0;
}
'''


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
def test_shifted_tiles_cover_the_grid(tmp_path):
    from nlsemagic_gb300 import build as B
    src = tmp_path / "ts.cu"
    src.write_text(SRC)
    exe = tmp_path / "ts"
    cmd = [B.nvcc()] + B.ARCH + ["-O2", "-std=c++17", "--extended-lambda", "-I", B.CSRC,
                                 "-I", B.INCLUDE, str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith("OK"), out.stdout + out.stderr
