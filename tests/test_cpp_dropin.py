"""The header-only C++ drop-in (include/dmsim/simulation.hpp) compiles against
the reference's example code shape, and on a GPU prints the adder's answer."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "dm-sim_gb300", "lib")


def build(tmp_path):
    exe = str(tmp_path / "adder_dropin")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "adder_dropin.cpp"), "-L", LIBDIR, "-ldmsim_gb300",
                           "-Wl,-rpath," + LIBDIR, "-o", exe])
    return exe


def test_dropin_header_compiles_and_links(engine, tmp_path):
    assert os.path.exists(build(tmp_path))


@pytest.mark.gpu
def test_dropin_adder_runs(engine, tmp_path):
    out = subprocess.run([build(tmp_path)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    shots = [ln.split(": ")[1] for ln in out.stdout.splitlines() if ln.startswith("Test-")]
    assert shots == ["1000000010"] * 5
