"""The XACC backend (include/dmsim/xacc_backend.hpp): the DmSimBackend
interface of the reference's XACC plugin (xacc/DmSimApi.hpp) and its
accelerator's execute() logic over the engine, checked on the reference's own
XACC test cases (xacc/tests/DmSimCpuAcceleratorTester.cpp) with XACC's IR
replaced by a plain instruction list (XACC is not installed here)."""
import os
import subprocess

import pytest

from test_known_answers import DEUTERON

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "dm-sim_gb300", "lib")


def build(tmp_path):
    exe = str(tmp_path / "xacc_backend_test")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "xacc_backend_test.cpp"), "-L", LIBDIR, "-ldmsim_gb300",
                           "-Wl,-rpath," + LIBDIR, "-o", exe])
    return exe


def test_xacc_backend_compiles_and_links(engine, tmp_path):
    assert os.path.exists(build(tmp_path))


def counts(line):
    return {kv.split(":")[0]: int(kv.split(":")[1]) for kv in line.split()[1:]}


@pytest.mark.gpu
def test_xacc_backend_reference_cases(engine, tmp_path):
    out = subprocess.run([build(tmp_path)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = {}
    deut = []
    for ln in out.stdout.splitlines():
        if ln.startswith("deuteron"):
            deut.append(float(ln.split()[2]))
        else:
            lines[ln.split()[0]] = ln
    # the reference's tolerance for 100000 shots
    assert len(deut) == 20 and all(abs(a - b) <= 0.01 for a, b in zip(deut, DEUTERON)), deut
    assert counts(lines["nothing"]) == {"00": 100}
    assert counts(lines["x_cx"]) == {"11": 100}
    bell = counts(lines["bell"])
    assert set(bell) <= {"00", "11"} and sum(bell.values()) == 100
    ch = counts(lines["ch"])  # X(0) then CH(0, 1): qubit 1 is |+>, not swapped
    assert set(ch) == {"10", "11"} and abs(ch["10"] - 10000) < 600, ch
    assert counts(lines["ccx"]) == {"7": 50}
    assert lines["all_ops"] == "all_ops 38"
