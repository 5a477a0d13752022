"""The FP64 issue rates the roofline rests on (tests/fp64_issue_rates.cu):
DADD and DMUL chains issue at the same rate, which is the rate
fgc_measure_fp64_rate reports, and a DFMA of three general register operands
issues faster (ncu's FP64 peak). Loose bounds: the test checks the ordering,
not a number."""
import ctypes
import os
import shutil
import subprocess

import pytest

from fauxgl_gb300 import _abi
from fauxgl_gb300 import build as B

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_fp64_issue_rates(tmp_path, gpu_lib):
    nvcc = B.nvcc()
    if not (os.path.isabs(nvcc) and os.path.exists(nvcc)) and shutil.which(nvcc) is None:
        pytest.skip("no nvcc")
    exe = str(tmp_path / "fp64_issue_rates")
    subprocess.run([nvcc] + B.ARCH + ["-O3", "--fmad=false", os.path.join(HERE, "fp64_issue_rates.cu"), "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
    rates = dict(line.split() for line in r.stdout.strip().splitlines()[:-1])
    dadd, dmul, dfma = float(rates["dadd"]), float(rates["dmul"]), float(rates["dfma"])
    assert 0.9 < dmul / dadd < 1.1
    assert dfma > 1.05 * dadd
    # the library's probe measures the add rate
    g = ctypes.c_double()
    _abi.check(gpu_lib.fgc_measure_fp64_rate(ctypes.byref(g)))
    assert 0.8 < (g.value / 32) / dadd < 1.25
