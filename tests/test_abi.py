"""The C-ABI library builds, loads and exports every entry point that
include/sgemtf.h declares.  No compute call: this runs without a GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "sgemtf.h")).read()
    return sorted(set(re.findall(r"^EMT_API [^(]*?\b(emt_\w+)\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("sgemtf_build",
                                                  os.path.join(ROOT, "sg-emtf_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    path = b.build()
    return ctypes.CDLL(path)


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s


def test_python_binding_lists_the_header(sgemtf):
    assert sorted(sgemtf.EXPORTED) == declared_symbols()


def test_config_default(sgemtf):
    c = sgemtf.Config()
    assert (c.algorithm, c.precision) == (sgemtf.DE_RAND1_BIN, sgemtf.ROT_FP32)
    assert (c.F, round(c.CR, 6), c.transfer_interval) == (0.5, 0.9, 0)
    assert c.p_m < 0  # 1/D


def test_reference_type_map(sgemtf, orc):
    L = sgemtf.lib()
    for t in range(-1, 8):
        assert L.emt_function_from_reference(t) == orc.lib().orc_function_from_reference(t)


def test_boxes_match_oracle(sgemtf, orc):
    for fid in range(7):
        for ref in (False, True):
            assert sgemtf.function_box(fid, ref) == orc.box(fid, ref)


def test_status_strings(sgemtf):
    for s in range(8):
        assert sgemtf.status_string(s)


def test_create_rejects_bad_config_before_touching_the_device(sgemtf):
    L = sgemtf.lib()
    h = ctypes.c_void_p()
    c = sgemtf.Config(algorithm=7)
    assert L.emt_create(ctypes.byref(c), ctypes.byref(h)) == sgemtf.ERR_INVALID_ARG
    c = sgemtf.Config(CR=1.5)
    assert L.emt_create(ctypes.byref(c), ctypes.byref(h)) == sgemtf.ERR_INVALID_ARG
    assert L.emt_create(None, ctypes.byref(h)) == sgemtf.ERR_INVALID_ARG
    assert L.emt_last_error(None) == b"null handle"
