"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/kmc_gb300.h (no GPU compute is called here)."""
import ctypes
import os
import re

import pytest

from coulomb_kmc_gb300 import _native

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "kmc_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(kmc_[a-z_]+)\s*\(", src)))


def test_library_builds_and_exports_header_symbols():
    path = _native.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(lib, s), s
    # the Python binding covers exactly the declared ABI
    assert set(_native.SIGNATURES) == set(syms)


def test_create_rejects_bad_parameters_without_gpu_work():
    lib = _native.lib()
    prm = _native.KmcParams()
    prm.boundary, prm.r, prm.l, prm.precision = 0, 1, 12, 0  # r < 2 is rejected before any CUDA call
    prm.extent, prm.max_move, prm.energy_unit = 4.0, 1.0, 1.0
    h = ctypes.c_void_p()
    assert lib.kmc_create(ctypes.byref(prm), ctypes.byref(h)) == -1
    assert h.value is None
    assert b"invalid" in lib.kmc_last_error()


def test_python_api_surface():
    import coulomb_kmc_gb300 as ck
    for name in ("initialise", "propose", "propose_with_dats", "accept", "free"):
        assert callable(getattr(ck.KMCFMM, name))
    with pytest.raises(NotImplementedError):
        ck.KMCFMM(ck.dats.PositionDat(4), ck.dats.ParticleDat(4), ck.dats.Domain(4.0),
                  boundary_condition="ff-only")


def test_host_propose_rejects_a_null_handle_without_gpu_work():
    lib = _native.lib()
    errs = (ctypes.c_int64 * 2)()
    assert lib.kmc_propose_with_dats_host(None, 1, 1, 1, None, None, None, None, None, None, errs) == -1
