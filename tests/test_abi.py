"""CPU tests of the C ABI: the library builds for sm_103a, loads, and exports
every entry point declared in include/*.h; argument checking happens before any
CUDA call, so it is exercised here without a GPU."""
import ctypes
import glob
import os
import re
import subprocess

import numpy as np

from zquatev_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        body = text.split('extern "C" {', 1)[1].split("} /* extern", 1)[0]
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", body):
            if m.group(1) not in ("if", "sizeof"):
                names.add(m.group(1))
    return names


def test_header_parsed():
    names = declared_functions()
    assert {"zquatev_c", "zquatev_device", "zq_stedc_device"} <= names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_reference_cxx_symbol_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert _lib.REFERENCE_SYMBOL in out
    fn = getattr(lib, _lib.REFERENCE_SYMBOL)
    assert fn(3, None, 4, None) == -1


def test_sm103a_code_in_library(lib):
    out = subprocess.run(["cuobjdump", "--list-elf", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "sm_103a" in out


def test_argument_errors(lib):
    d = np.zeros((4, 4), dtype=np.complex128, order="F")
    e = np.zeros(4)
    assert lib.zquatev_c(3, d.ctypes.data, 4, e.ctypes.data) == -1
    assert lib.zquatev_c(-2, d.ctypes.data, 4, e.ctypes.data) == -1
    assert lib.zquatev_c(4, None, 4, e.ctypes.data) == -2
    assert lib.zquatev_c(4, d.ctypes.data, 3, e.ctypes.data) == -3
    assert lib.zquatev_c(4, d.ctypes.data, 4, None) == -4
    assert lib.zquatev_c(0, None, 1, None) == 0
    assert "ld2" in _lib.last_error() or "null" in _lib.last_error() or _lib.last_error() == ""
    assert lib.zq_set_block_size(0) == -5
    assert lib.zq_set_block_size(129) == -5
    nb0 = lib.zq_get_block_size()
    assert lib.zq_set_block_size(32) == 0 and lib.zq_get_block_size() == 32
    assert lib.zq_set_block_size(nb0) == 0
    assert lib.zq_stedc_device(-1, None, None, None, None, 1, None) == -5
    n2s = (ctypes.c_int * 1)(3)
    assert lib.zquatev_batched_device(1, n2s, n2s, None, None, None, None, None) == -5


def test_python_mirror_validates_layout():
    from zquatev_gb300 import solver

    d = np.zeros((4, 4), dtype=np.complex128)  # C order: rejected
    try:
        solver.zquatev(4, d, 4, np.zeros(4))
    except TypeError:
        pass
    else:
        raise AssertionError("C-ordered D accepted")
