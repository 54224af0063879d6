"""The mixed-precision 3D interior kernel is compiled for 4 resident CTAs per
SM (64 registers); a register spill there costs far more than it saves, so
the build must report none (checked with ptxas, no GPU needed).  This
covers both interior kernels (one plane per iteration and two) and the 2D
single-pass stage kernel."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
def test_interior_kernel_does_not_spill(tmp_path):
    from nlsemagic_gb300 import build as B
    src = os.path.join(B.CSRC, "kern_mixed.cu")
    cmd = [B.nvcc()] + B.ARCH + B.COMMON + B.UNITS["kern_mixed.cu"] + \
        ["-Xptxas", "-v", "-c", src, "-o", str(tmp_path / "k.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    blocks = re.split(r"Compiling entry function '", r.stderr)
    seen = 0
    for b in blocks[1:]:
        name = b.split("'", 1)[0]
        if "wide6wide3d" not in name and "wide9wide3d_z2" not in name and \
                "wide2d7stage2d" not in name:
            continue
        seen += 1
        m = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", b)
        assert m and m.group(1) == "0" and m.group(2) == "0", (name, m.group(0) if m else b[:200])
    # 2 methods x 4 stages x TMA / plain loads, the two-plane form's
    # 2 methods x 4 stages x 3 tile heights, and the 2D kernel's 2 methods x
    # 3 codes x 4 stages x 3 tile heights
    assert seen == 112
