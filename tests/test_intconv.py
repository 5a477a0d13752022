"""The integer-pipe float64 conversions used by the setup and raster kernels
(fgc_intconv.cuh: Go's int(f), int(Floor/Ceil(f)), small int -> float64,
sign tests), compiled for the host, against the C library on seeded and
edge values."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_conversions_match_the_fp64_instructions(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "intconv_check")
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-std=c++17", os.path.join(HERE, "intconv_check.cpp"), "-o",
                    exe], check=True)
    r = subprocess.run([exe, "300000"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
