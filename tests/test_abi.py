"""The C-ABI library builds, loads and exports every entry point that
include/fastsht.h declares; argument validation works without a GPU."""
import ctypes as C
import re
from pathlib import Path

import pytest

from fastsht_gb300 import _lib, build

HEADER = Path(__file__).resolve().parent.parent / "include" / "fastsht.h"


def declared_functions():
    txt = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*int\s+(fsht_\w+)\s*\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    for want in ("fsht_plan_create", "fsht_plan_destroy", "fsht_t2alm", "fsht_alm2t",
                 "fsht_qu2eb", "fsht_eb2qu", "fsht_last_error"):
        assert want in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(lib):
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


@pytest.mark.parametrize("args,code", [
    ((3, 8, 1, 0, 0), _lib.FSHT_EINVAL),          # nside not a power of two
    ((0, 8, 1, 0, 0), _lib.FSHT_EINVAL),
    ((8, 33, 1, 0, 0), _lib.FSHT_EINVAL),         # lmax > 4 nside
    ((8, -1, 1, 0, 0), _lib.FSHT_EINVAL),
    ((8, 16, 0, 0, 0), _lib.FSHT_EINVAL),         # nmaps_max < 1
    ((4096, 100, 1, 0, 0), _lib.FSHT_EUNSUPPORTED),   # above nside 2048
    ((8, 16, 1, 0, 7), _lib.FSHT_EUNSUPPORTED),   # unknown precision
])
def test_plan_create_rejects_bad_arguments(lib, args, code):
    plan = C.c_void_p()
    rc = lib.fsht_plan_create(*args, 0, None, C.byref(plan))
    assert rc == code
    assert plan.value is None
    assert len(_lib.last_error()) > 0


def test_null_plan_is_an_error(lib):
    rc = lib.fsht_t2alm(None, None, None, 1, 0, 0)
    assert rc == _lib.FSHT_EINVAL
    assert "plan" in _lib.last_error()


def test_host_mapped_without_library_blocks(lib):
    """Memory that fsht_host_alloc did not return is never read in place (no CUDA call is
    needed to say so); a null output pointer is an argument error."""
    import numpy as np
    a = np.zeros(1000)
    m = C.c_int(-1)
    assert lib.fsht_host_mapped(C.c_void_p(a.ctypes.data), C.c_size_t(a.nbytes), C.byref(m)) == 0
    assert m.value == 0
    assert lib.fsht_host_mapped(None, C.c_size_t(8), C.byref(m)) == 0
    assert m.value == 0
    assert lib.fsht_host_mapped(C.c_void_p(a.ctypes.data), C.c_size_t(8), None) == _lib.FSHT_EINVAL


def test_host_read_setter_needs_a_plan(lib):
    assert lib.fsht_plan_set_host_read(None, 1) == _lib.FSHT_EINVAL
    assert "plan" in _lib.last_error()


@pytest.mark.parametrize("nside,lmax,code", [
    (512, 168, _lib.FSHT_EUNSUPPORTED),    # tables + one map above the fixed scratch
    (1024, 64, _lib.FSHT_EUNSUPPORTED),
    (2048, 64, _lib.FSHT_EUNSUPPORTED),    # half-length ring transforms: plan path only
    (3, 8, _lib.FSHT_EINVAL),              # not a power of two
    (8, 33, _lib.FSHT_EINVAL),             # lmax > 4 nside
])
def test_noalloc_rejects_sizes_before_any_device_work(lib, nside, lmax, code):
    """The allocation-free analysis checks its size rule on the host first: these sizes are
    refused without touching a device (the pointers are never used)."""
    rc = lib.fsht_t2alm_noalloc(nside, lmax, C.c_void_p(16), C.c_void_p(16), 1, None)
    assert rc == code
    assert len(_lib.last_error()) > 0


def test_range_status_is_declared():
    assert "FSHT_ERANGE = -6" in HEADER.read_text()
    assert _lib.FSHT_ERANGE == -6
