"""The split form's forward ring FFT (df64 arithmetic on the FP32 pipe) against the FP64 one.

Both plans run FSHT_STAGE_FFT_FWD on the same maps; the {S, D} phase matrices must agree to
1e-12 of each map's largest entry (df64 carries ~48 significand bits; the FP64 transform is the
one the oracle pins).  Cases cover power-of-two, Bluestein 2^k and 3*2^k rings, the
half-length rings of nside 2048, all-zero maps and values far outside FP32's range."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

DF_TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastsht_gb300 import build
    build.build()


def _fft_stage(ns, lmax, maps, precision):
    from fastsht_gb300 import _lib
    nmaps = maps.shape[0]
    plan = C.c_void_p()
    _lib.call("fsht_plan_create", ns, lmax, nmaps, 0, precision, 0, None, C.byref(plan))
    try:
        W = torch.zeros((lmax + 1, 2 * ns, nmaps, 2, 2), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _lib.call("fsht_run_stage", plan, 0, C.c_void_p(maps.data_ptr()),
                  C.c_void_p(W.data_ptr()), nmaps)
        _lib.call("fsht_plan_sync", plan)
        return W
    finally:
        _lib.load().fsht_plan_destroy(plan)


def _rel_err(ns, lmax, maps):
    from fastsht_gb300 import _lib
    w64 = _fft_stage(ns, lmax, maps, _lib.FSHT_PREC_FP64)
    wdf = _fft_stage(ns, lmax, maps, _lib.FSHT_PREC_SPLIT)
    assert torch.isfinite(wdf).all()
    d = (wdf - w64).abs().amax(dim=(0, 1, 3, 4))
    ref = w64.abs().amax(dim=(0, 1, 3, 4))
    ok = ref > 0
    assert torch.equal(d[~ok], torch.zeros_like(d[~ok])), "all-zero maps must give zeros"
    return float((d[ok] / ref[ok]).max()) if ok.any() else 0.0


@pytest.mark.parametrize("ns,lmax,nmaps", [(1, 3, 2), (2, 5, 3), (4, 11, 3), (16, 47, 5),
                                           (64, 191, 7), (256, 767, 3), (1024, 2047, 2)])
def test_df_fft_matches_fp64(ns, lmax, nmaps):
    g = torch.Generator(device="cuda").manual_seed(ns + nmaps)
    maps = torch.randn((nmaps, 12 * ns * ns), dtype=torch.float64, device="cuda", generator=g)
    assert _rel_err(ns, lmax, maps) <= DF_TOL


def test_df_fft_half_length_rings_nside_2048():
    ns, lmax = 2048, 4096
    g = torch.Generator(device="cuda").manual_seed(5)
    maps = torch.randn((1, 12 * ns * ns), dtype=torch.float64, device="cuda", generator=g)
    assert _rel_err(ns, lmax, maps) <= DF_TOL


def test_df_fft_scales_and_zeros():
    """Per-(ring pair, map) power-of-two scaling: 1e-200 / 1e+200 maps keep the relative
    accuracy, an all-zero map gives exact zeros, one hot pixel per map is exact-ish."""
    ns, lmax = 32, 95
    npix = 12 * ns * ns
    g = torch.Generator(device="cuda").manual_seed(7)
    base = torch.randn((5, npix), dtype=torch.float64, device="cuda", generator=g)
    base[0] *= 1e-200
    base[1] *= 1e200
    base[2] = 0.0
    base[3, 1000:] = 0.0
    base[3, :1000] *= 1e-3
    base[4] = 0.0
    base[4, 4321] = 3.0
    assert _rel_err(ns, lmax, base) <= DF_TOL


def test_df_fft_wide_dynamic_range_within_a_ring():
    """Values spanning 1e-30..1 inside one ring: the error stays relative to the ring maximum."""
    ns, lmax = 16, 47
    npix = 12 * ns * ns
    g = torch.Generator(device="cuda").manual_seed(9)
    m = torch.randn((2, npix), dtype=torch.float64, device="cuda", generator=g)
    m *= torch.logspace(-30, 0, npix, dtype=torch.float64, device="cuda")
    assert _rel_err(ns, lmax, m) <= DF_TOL


def _inv_stage(ns, lmax, W, precision):
    from fastsht_gb300 import _lib
    nmaps = W.shape[2]
    plan = C.c_void_p()
    _lib.call("fsht_plan_create", ns, lmax, nmaps, 0, precision, 0, None, C.byref(plan))
    try:
        maps = torch.zeros((nmaps, 12 * ns * ns), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _lib.call("fsht_run_stage", plan, 3, C.c_void_p(W.data_ptr()),
                  C.c_void_p(maps.data_ptr()), nmaps)
        _lib.call("fsht_plan_sync", plan)
        return maps
    finally:
        _lib.load().fsht_plan_destroy(plan)


@pytest.mark.parametrize("ns,lmax,nmaps", [(1, 3, 2), (4, 11, 3), (16, 47, 5), (64, 191, 4),
                                           (256, 767, 2), (1024, 2047, 1), (2048, 4096, 1)])
def test_df_inverse_fft_matches_fp64(ns, lmax, nmaps):
    """FSHT_STAGE_FFT_INV (the synthesis side: aliased spectrum from {G_N, G_S}, inverse ring
    DFT) of the same random phase matrix; maps agree to 1e-12 of each map's largest pixel."""
    from fastsht_gb300 import _lib
    g = torch.Generator(device="cuda").manual_seed(3 * ns + nmaps)
    W = torch.randn((lmax + 1, 2 * ns, nmaps, 2, 2), dtype=torch.float64, device="cuda",
                    generator=g)
    if nmaps > 1:
        W[:, :, 1] *= 1e-120                           # a map far below FP32's range
    m64 = _inv_stage(ns, lmax, W, _lib.FSHT_PREC_FP64)
    mdf = _inv_stage(ns, lmax, W, _lib.FSHT_PREC_SPLIT)
    assert torch.isfinite(mdf).all()
    d = (mdf - m64).abs().amax(dim=1)
    ref = m64.abs().amax(dim=1)
    assert float((d / ref).max()) <= DF_TOL
