"""The vertex stage's division by W through the correctly rounded reciprocal
(div_by_rcp in fauxgl_gb300/csrc/fgc_device.cuh) against __ddiv_rn on the
GPU, bit for bit, over ~300 M seeded operand pairs (tests/divrcp_check.cu)."""
import os
import shutil
import subprocess

import pytest

from fauxgl_gb300 import build as B

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_division_by_reciprocal_matches_the_division(tmp_path):
    nvcc = B.nvcc()
    if not (os.path.isabs(nvcc) and os.path.exists(nvcc)) and shutil.which(nvcc) is None:
        pytest.skip("no nvcc")
    exe = str(tmp_path / "divrcp_check")
    subprocess.run([nvcc] + B.ARCH + ["-O3", "--fmad=false", "-std=c++17", os.path.join(HERE, "divrcp_check.cu"),
                                      "-o", exe], check=True)
    r = subprocess.run([exe, "256"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
