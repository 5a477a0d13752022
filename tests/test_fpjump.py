"""The exact k-fold FP64 sum used by the raster stage (fgc_fpjump.cuh),
compiled for the host, against the plain loop on seeded adversarial cases."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_repeat_add_matches_the_serial_loop(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "fpjump_check")
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-std=c++17", os.path.join(HERE, "fpjump_check.cpp"), "-o", exe],
                   check=True)
    r = subprocess.run([exe, "400000"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
