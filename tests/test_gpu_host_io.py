"""Host-buffer analysis (fsht_t2alm_host, used by SHT.t2alm for NumPy inputs): the maps go to
the device in sub-batches that the FFT consumes as they land and alm columns come back as waves
finish.  The results must equal the device-buffer path bit for bit, for both precisions, with
refinement, with several workspace chunks, into a caller's output array and from pageable
(not pinned) input."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastsht_gb300 import build
    build.build()


def _maps(ns, nsim, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal((12 * ns * ns, nsim)))


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("niter", [0, 1])
def test_host_path_equals_device_path(precision, niter):
    from fastsht_gb300 import SHT
    ns, lmax, nsim = 64, 191, 70
    maps = _maps(ns, nsim, 1)
    sht = SHT(ns, lmax, nsim, niter=niter, precision=precision)
    got = sht.t2alm(maps)                                     # host in, host out
    dev = torch.from_numpy(maps.T.copy()).cuda().T            # (npix, nsim) Fortran view
    want = sht.t2alm(dev).cpu().numpy()
    assert isinstance(got, np.ndarray) and got.shape == (nsim, lmax + 1, lmax + 1)
    assert np.array_equal(got, want)
    assert np.array_equal(sht.get_alms(), want)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_host_path_several_chunks_and_caller_output(precision):
    from fastsht_gb300 import SHT
    ns, lmax, nsim = 64, 191, 150
    maps = _maps(ns, nsim, 2)
    # the split plan's fixed part: two lambda staging and two digit-tile buffers (~220 MB here)
    sht = SHT(ns, lmax, nsim, precision=precision,
              workspace_limit=(60 << 20) if precision == "fp64" else (300 << 20))
    assert sht.plan_info()["maps_per_chunk"] < nsim
    out = np.zeros((nsim, lmax + 1, lmax + 1), order="F")
    assert sht.t2alm(maps, alms_in=out) == 0
    want = sht.t2alm(torch.from_numpy(maps.T.copy()).cuda().T).cpu().numpy()
    assert np.array_equal(out, want)


def test_host_path_split_nside_1024():
    """The headline shape class (17 waves, per-wave column returns), 3 maps."""
    from fastsht_gb300 import SHT
    ns, lmax, nsim = 1024, 2047, 3
    maps = _maps(ns, nsim, 3)
    sht = SHT(ns, lmax, nsim, precision="split")
    got = sht.t2alm(maps)
    want = sht.t2alm(torch.from_numpy(maps.T.copy()).cuda().T).cpu().numpy()
    assert np.array_equal(got, want)


def test_pinned_empty_buffers():
    """Library-allocated page-locked buffers (fsht_host_alloc) as t2alm input and output."""
    from fastsht_gb300 import SHT, pinned_empty
    ns, lmax, nsim = 32, 95, 5
    sht = SHT(ns, lmax, nsim, precision="split")
    maps = pinned_empty((12 * ns * ns, nsim))
    maps[...] = _maps(ns, nsim, 4)
    out = pinned_empty((nsim, lmax + 1, lmax + 1))
    assert out.flags.f_contiguous and maps.flags.f_contiguous
    assert sht.t2alm(maps, alms_in=out) == 0
    want = sht.t2alm(torch.from_numpy(np.asarray(maps).T.copy()).cuda().T).cpu().numpy()
    assert np.array_equal(out, want)
    del maps, out                                  # freed through fsht_host_free


def _mapped(ptr, nbytes):
    import ctypes as C
    from fastsht_gb300 import _lib
    m = C.c_int(-1)
    _lib.call("fsht_host_mapped", C.c_void_p(ptr), C.c_size_t(nbytes), C.byref(m))
    return m.value


def test_host_mapped_ranges():
    """Only byte ranges inside one fsht_host_alloc block are read in place."""
    from fastsht_gb300 import pinned_empty
    buf = pinned_empty((1000,))
    p = buf.ctypes.data
    assert _mapped(p, buf.nbytes) == 1
    assert _mapped(p + 800, 200 * 8) == 1
    assert _mapped(p + 8, buf.nbytes) == 0          # one double past the block's end
    assert _mapped(np.zeros(1000).ctypes.data, 8000) == 0   # pageable memory
    del buf
    assert _mapped(p, 8000) == 0                    # freed blocks are forgotten


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("niter", [0, 1])
def test_direct_read_equals_staged_and_device_paths(precision, niter):
    """Maps in a pinned_empty buffer, read in place by the FFT (the default) and copied first
    (host_read="staged"): both equal the device-buffer path bit for bit."""
    from fastsht_gb300 import SHT, pinned_empty
    ns, lmax, nsim = 64, 191, 70
    maps = pinned_empty((12 * ns * ns, nsim))
    maps[...] = _maps(ns, nsim, 5)
    assert _mapped(maps.ctypes.data, maps.nbytes) == 1
    want = SHT(ns, lmax, nsim, niter=niter, precision=precision).t2alm(
        torch.from_numpy(np.asarray(maps).T.copy()).cuda().T).cpu().numpy()
    direct = SHT(ns, lmax, nsim, niter=niter, precision=precision)
    got = direct.t2alm(maps)
    assert direct._host_dev[0] is None              # no device staging buffer for the maps
    staged = SHT(ns, lmax, nsim, niter=niter, precision=precision, host_read="staged")
    got_s = staged.t2alm(maps)
    assert staged._host_dev[0] is not None
    assert np.array_equal(got, want)
    assert np.array_equal(got_s, want)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_direct_read_several_chunks_nside_1024(precision):
    """In-place reads with several workspace chunks, and the headline shape class."""
    from fastsht_gb300 import SHT, pinned_empty
    for ns, lmax, nsim, lim in [(64, 191, 150, (60 << 20) if precision == "fp64" else (300 << 20)),
                                (1024, 2047, 2, 0)]:
        maps = pinned_empty((12 * ns * ns, nsim))
        maps[...] = _maps(ns, nsim, 6)
        sht = SHT(ns, lmax, nsim, precision=precision, workspace_limit=lim)
        if lim:
            assert sht.plan_info()["maps_per_chunk"] < nsim
        got = sht.t2alm(maps)
        want = sht.t2alm(torch.from_numpy(np.asarray(maps).T.copy()).cuda().T).cpu().numpy()
        assert np.array_equal(got, want)
        sht.close()
        del maps


def test_chunked_direct_read_equals_device_path():
    """The split form's chunked in-place route (128-map chunks, each chunk's contraction beside
    the next chunk's host reads, two phase-matrix buffers alternating) gives the device path's
    alm bit for bit, as does the one-chunk route (the default)."""
    from fastsht_gb300 import SHT, pinned_empty
    ns, lmax, nsim = 64, 191, 300
    maps = pinned_empty((12 * ns * ns, nsim))
    maps[...] = _maps(ns, nsim, 8)
    want = SHT(ns, lmax, nsim, precision="split").t2alm(
        torch.from_numpy(np.asarray(maps).T.copy()).cuda().T).cpu().numpy()
    for mode in ("direct_chunked", "direct"):
        sht = SHT(ns, lmax, nsim, precision="split", host_read=mode)
        got = sht.t2alm(maps)
        got2 = sht.t2alm(maps)                      # buffers reused on a second call
        assert np.array_equal(got, want), mode
        assert np.array_equal(got2, want), mode
        sht.close()
