"""fsht_t2alm_noalloc: the allocation-free temperature analysis.

It serves callers that may not allocate device memory where they transform
(their host application owns the device memory, or an allocation would stall a
latency-critical loop).  Checked through the C ABI against the plan-based
fsht_t2alm on the same device inputs, on two calls in a row (the second call
reuses the library's fixed scratch array left over from the first).  This file is
collected last so that a stopping run has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = 1e-11


def _rel(a, b):
    """max |a - b| / max |b| per map (first axis), then the max over maps."""
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    d = np.abs(a - b).max(axis=1)
    s = np.abs(b).max(axis=1)
    return float((d / s).max())


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastsht_gb300 import _lib, build
    build.build()
    return _lib


@pytest.mark.parametrize("nside,lmax,nmaps", [(8, 23, 3), (64, 191, 12), (256, 1024, 3),
                                              (512, 167, 2)])
def test_noalloc_matches_plan_path_twice(lib, nside, lmax, nmaps):
    from fastsht_gb300 import SHT
    rng = np.random.default_rng(nside)
    npix = 12 * nside * nside
    L = lmax + 1
    maps = torch.from_numpy(rng.standard_normal((nmaps, npix))).cuda()
    want = SHT(nside, lmax, nmaps).t2alm(maps.T)                 # (nmaps, L, L) device view
    want = want.permute(2, 1, 0).contiguous().cpu().numpy()     # (L, L, nmaps)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        alm = torch.full((L, L, nmaps), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        lib.call("fsht_t2alm_noalloc", nside, lmax, C.c_void_p(maps.data_ptr()),
                 C.c_void_p(alm.data_ptr()), nmaps, C.c_void_p(stream))
        torch.cuda.synchronize()
        if call == 1:
            # the point of the entry point: once its kernels are loaded (first call), a call
            # takes no device memory at all
            assert torch.cuda.mem_get_info()[0] == free_before
        got = alm.cpu().numpy()
        assert np.isfinite(got).all()
        err = _rel(np.moveaxis(got, 2, 0), np.moveaxis(want, 2, 0))
        assert err <= TOL, (call, err)


def test_noalloc_rejects_sizes_above_its_scratch(lib):
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    with pytest.raises(lib.FshtError) as ei:
        lib.call("fsht_t2alm_noalloc", 512, 2048, C.c_void_p(x.data_ptr()),
                 C.c_void_p(x.data_ptr()), 1, None)
    assert ei.value.code == lib.FSHT_EUNSUPPORTED
    assert "static scratch" in str(ei.value)
    with pytest.raises(lib.FshtError) as ei:
        lib.call("fsht_t2alm_noalloc", 2048, 64, C.c_void_p(x.data_ptr()),
                 C.c_void_p(x.data_ptr()), 1, None)
    assert ei.value.code == lib.FSHT_EUNSUPPORTED
    with pytest.raises(ValueError):
        lib.call("fsht_t2alm_noalloc", 12, 8, C.c_void_p(x.data_ptr()),
                 C.c_void_p(x.data_ptr()), 1, None)
