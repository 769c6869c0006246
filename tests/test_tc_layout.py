"""The tensor-core tile layout's safety property, on the host: every MMA of
an island's rotation reads inside the launch's shared memory and every TMA
copy of Q lands inside the B region (emt::tc_island_reads_inside, which the
library also checks before a tensor-core launch), over island shapes across
the supported range.  Compiles tests/cpp/tc_layout_check.cpp with g++ against
the library's internal header; no GPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_mma_reads_stay_inside_the_allocation(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "tc_layout_check")
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "sg-emtf_gb300", "csrc"),
                        os.path.join(HERE, "cpp", "tc_layout_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 outside" in r.stdout
