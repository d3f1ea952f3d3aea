"""The C-ABI library loads and exports every entry point include/*.h declares;
argument checks that need no GPU behave."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        syms |= set(re.findall(r"^\s*(?:const\s+char\s*\*|int)\s+(dmsim_\w+)\s*\(", txt, re.M))
    return sorted(syms)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("dmsim_create", "dmsim_append", "dmsim_upload", "dmsim_run", "dmsim_measure", "dmsim_get_dm"):
        assert s in syms


@pytest.mark.parametrize("sym", declared_symbols())
def test_library_exports(engine, sym):
    assert hasattr(engine.lib(), sym), sym


def test_multi_gpu_request_is_unsupported_not_fatal(engine):
    h = ctypes.c_void_p()
    assert engine.lib().dmsim_create(4, 2, ctypes.byref(h)) == engine.ERR_UNSUPPORTED
    assert engine.lib().dmsim_create(0, 1, ctypes.byref(h)) == engine.ERR_ARG
    assert engine.lib().dmsim_status_string(engine.ERR_CUDA) == b"CUDA error"


def test_null_handle_is_an_error(engine):
    assert engine.lib().dmsim_run(None) == engine.ERR_ARG
    assert engine.lib().dmsim_upload(None) == engine.ERR_ARG
