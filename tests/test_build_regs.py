"""The mixed-precision 3D interior kernel is compiled for 4 resident CTAs per
SM (64 registers); a register spill there costs far more than it saves, so
the build must report none (checked with ptxas, no GPU needed).  Both forms
are checked: the interior kernel of the three-kernel form (kern_mixed.cu)
and the kernel with the face work fused in (kern_wfuse.cu)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ptxas_blocks(unit, tmp_path):
    from nlsemagic_gb300 import build as B
    src = os.path.join(B.CSRC, unit)
    cmd = [B.nvcc()] + B.ARCH + B.COMMON + B.UNITS[unit] + \
        ["-Xptxas", "-v", "-c", src, "-o", str(tmp_path / "k.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = []
    for b in re.split(r"Compiling entry function '", r.stderr)[1:]:
        name = b.split("'", 1)[0]
        if "wide6wide3d" in name:
            out.append((name, b))
    return out


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
@pytest.mark.parametrize("unit,count", [
    ("kern_mixed.cu", 16),  # 2 methods x 4 stages x TMA / plain loads
    ("kern_wfuse.cu", 24),  # 3 boundary codes x 4 stages x TMA / plain loads
])
def test_interior_kernel_does_not_spill(tmp_path, unit, count):
    blocks = _ptxas_blocks(unit, tmp_path)
    for name, b in blocks:
        m = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", b)
        assert m and m.group(1) == "0" and m.group(2) == "0", (name, m.group(0) if m else b[:200])
        regs = re.search(r"Used (\d+) registers", b)
        assert regs and int(regs.group(1)) <= 64, (name, regs.group(0) if regs else "")
    assert len(blocks) == count
