"""Host check of the tensor-core pass descriptors (CPU): tile geometry,
run masks and the BF16 operator slices of 1400+ passes from random circuits
(tests/cpp/tc_desc_check.cpp, compiled against the planner's sources)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dm-sim_gb300", "csrc")


def test_tensor_descriptors(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "tc_desc_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "tc_desc_check.cpp"), os.path.join(CSRC, "plan.cpp"),
                    os.path.join(CSRC, "gates.cpp"), "-o", exe], check=True, capture_output=True, text=True,
                   timeout=300)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
