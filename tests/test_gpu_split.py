"""The split-precision form (BF16 slice products on tcgen05) against the FP64
oracle.  Bar: max_{l,m}|a - a_fp64| / max|a_fp64| <= 1e-7 per map (the precision
target); the FP64 path is the oracle-pinned reference here."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import rel_alm_err
from oracle import OracleSHT, gaussian_alm

pytestmark = pytest.mark.gpu

SPLIT_TOL = 1e-7


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastsht_gb300 import build
    build.build()


def SHT(*a, **k):
    from fastsht_gb300 import SHT as _S
    return _S(*a, **k)


def bandlimited_maps(ns, lmax, nsim, seed):
    rng = np.random.default_rng(seed)
    l = np.arange(lmax + 1, dtype=float)
    cl = 1.0 / np.maximum(l, 1.0) ** 2
    cl[0] = 0
    alm = gaussian_alm(cl, lmax, nsim, rng)
    return SHT(ns, lmax, nsim).alm2t(alm)


@pytest.mark.parametrize("ns,lmax,nsim", [(4, 11, 2), (8, 23, 3), (16, 47, 5), (64, 191, 100),
                                          (64, 128, 130), (128, 383, 9)])
def test_split_t2alm_matches_oracle(ns, lmax, nsim):
    maps = bandlimited_maps(ns, lmax, nsim, ns + nsim)
    sht = SHT(ns, lmax, nsim, precision="split")
    got = sht.t2alm(maps)
    want = OracleSHT(ns, lmax, ring_tab=sht.ring_skip()).t2alm(maps)
    err = rel_alm_err(got, want)
    assert err <= SPLIT_TOL, err


def test_split_white_noise_maps():
    """Unstructured N(0,1) pixels (config-1 style inputs) also meet the bar."""
    ns, lmax, nsim = 32, 95, 6
    rng = np.random.default_rng(0)
    maps = np.asfortranarray(rng.standard_normal((12 * ns * ns, nsim)))
    sht = SHT(ns, lmax, nsim, precision="split")
    got = sht.t2alm(maps)
    want = OracleSHT(ns, lmax, ring_tab=sht.ring_skip()).t2alm(maps)
    assert rel_alm_err(got, want) <= SPLIT_TOL


def test_split_matches_fp64_path_at_nside_1024():
    """nside 1024 / lmax 2047 (the precision-form config), 4 maps: split vs plain."""
    ns, lmax, nsim = 1024, 2047, 4
    maps = bandlimited_maps(ns, lmax, nsim, 2)
    a64 = SHT(ns, lmax, nsim).t2alm(maps)
    a16 = SHT(ns, lmax, nsim, precision="split").t2alm(maps)
    assert rel_alm_err(a16, a64) <= SPLIT_TOL


def rel_map_err(a, b):
    """max over maps of max_pix |a - b| / max_pix |b| ((npix, nsim) arrays)."""
    d = np.abs(np.asarray(a) - np.asarray(b)).max(axis=0)
    return float((d / np.abs(np.asarray(b)).max(axis=0)).max())


def _alm(lmax, nsim, seed):
    rng = np.random.default_rng(seed)
    l = np.arange(lmax + 1, dtype=float)
    cl = 1.0 / np.maximum(l, 1.0) ** 2
    cl[0] = 0
    return gaussian_alm(cl, lmax, nsim, rng)


@pytest.mark.parametrize("ns,lmax,nsim", [(4, 11, 2), (16, 47, 5), (64, 191, 70), (128, 300, 3)])
def test_split_alm2t_matches_oracle(ns, lmax, nsim):
    """Split synthesis (lambda against one global scale, alm digits per column) against
    the FP64 oracle's alm2map."""
    alm = _alm(lmax, nsim, ns + 7)
    sht = SHT(ns, lmax, nsim, precision="split")
    got = sht.alm2t(alm)
    want = OracleSHT(ns, lmax, ring_tab=sht.ring_skip()).alm2t(alm)
    assert rel_map_err(got, want) <= SPLIT_TOL


def test_split_alm2t_l_chunks_at_lmax_2048():
    """lmax 2048: 1025 l of even parity at m = 0, so l-chunks add into the phase matrix."""
    ns, lmax, nsim = 512, 2048, 2
    alm = _alm(lmax, nsim, 11)
    m64 = SHT(ns, lmax, nsim).alm2t(alm)
    m16 = SHT(ns, lmax, nsim, precision="split").alm2t(alm)
    assert rel_map_err(m16, m64) <= SPLIT_TOL


@pytest.mark.parametrize("method", ["old", "new"])
@pytest.mark.parametrize("niter", [1, 2])
def test_split_refinement_matches_fp64_iterations(niter, method):
    """niter Jacobi refinement steps in the split form (split synthesis and analysis, FP64
    Fourier-space residual) against the plain path with the same niter and method."""
    ns, lmax, nsim = 64, 191, 6
    maps = bandlimited_maps(ns, lmax, nsim, 5)
    a64 = SHT(ns, lmax, nsim, niter=niter).t2alm(maps, method=method)
    a16 = SHT(ns, lmax, nsim, niter=niter, precision="split").t2alm(maps, method=method)
    assert rel_alm_err(a16, a64) <= SPLIT_TOL
    # the refinement changes the result as the plain iteration does: the round-trip
    # residual of the split form equals the plain one's
    back = SHT(ns, lmax, nsim)
    r16 = np.abs(back.alm2t(a16) - maps).max()
    r64 = np.abs(back.alm2t(a64) - maps).max()
    r0 = np.abs(back.alm2t(SHT(ns, lmax, nsim).t2alm(maps)) - maps).max()
    assert abs(r16 - r64) <= 1e-6 * r64 and abs(r64 - r0) > 1e-3 * r0


def test_split_refinement_at_nside_1024():
    """One refinement step at the precision-form config size (4 maps)."""
    ns, lmax, nsim = 1024, 2047, 4
    maps = bandlimited_maps(ns, lmax, nsim, 2)
    a64 = SHT(ns, lmax, nsim, niter=1).t2alm(maps)
    a16 = SHT(ns, lmax, nsim, niter=1, precision="split").t2alm(maps)
    assert rel_alm_err(a16, a64) <= SPLIT_TOL


def _pol_maps(ns, lmax, nsim, seed):
    rng = np.random.default_rng(seed)
    l = np.arange(lmax + 1, dtype=float)
    cl = np.where(l >= 2, 1.0 / np.maximum(l * (l + 1), 1.0), 0.0)
    E = gaussian_alm(cl, lmax, nsim, rng)
    B = gaussian_alm(0.1 * cl, lmax, nsim, rng)
    return SHT(ns, lmax, nsim, pol=True).eb2qu(E, B)


@pytest.mark.parametrize("ns,lmax,nsim", [(4, 11, 2), (16, 47, 5), (64, 191, 70), (128, 300, 3)])
def test_split_qu2eb_matches_fp64(ns, lmax, nsim):
    """Spin-2 split analysis (lambda1/lambda2 digit products, the +-i routing) against the
    plain path, E and B each within the bar."""
    Q, U = _pol_maps(ns, lmax, nsim, ns + 3)
    E64, B64 = SHT(ns, lmax, nsim, pol=True).qu2eb(Q, U)
    sht = SHT(ns, lmax, nsim, pol=True, precision="split")
    E16, B16 = sht.qu2eb(Q, U)
    assert rel_alm_err(E16, E64) <= SPLIT_TOL
    assert rel_alm_err(B16, B64) <= SPLIT_TOL
    assert rel_alm_err(sht.qu2e(Q, U), E64) <= SPLIT_TOL
    assert rel_alm_err(sht.qu2b(Q, U), B64) <= SPLIT_TOL


def test_split_qu2eb_ring_chunks_at_nside_1024():
    """nside 1024: 2048 north rings, so ring K-chunks add into E/B with atomics."""
    ns, lmax, nsim = 1024, 2047, 2
    Q, U = _pol_maps(ns, lmax, nsim, 9)
    E64, B64 = SHT(ns, lmax, nsim, pol=True).qu2eb(Q, U)
    E16, B16 = SHT(ns, lmax, nsim, pol=True, precision="split").qu2eb(Q, U)
    assert rel_alm_err(E16, E64) <= SPLIT_TOL
    assert rel_alm_err(B16, B64) <= SPLIT_TOL


def test_split_qu2eb_refinement():
    """niter = 1 on Q/U: FP64 spin-2 synthesis and residual, split analyses."""
    ns, lmax, nsim = 32, 80, 4
    Q, U = _pol_maps(ns, lmax, nsim, 10)
    E64, B64 = SHT(ns, lmax, nsim, niter=1, pol=True).qu2eb(Q, U)
    E16, B16 = SHT(ns, lmax, nsim, niter=1, pol=True, precision="split").qu2eb(Q, U)
    assert rel_alm_err(E16, E64) <= SPLIT_TOL
    assert rel_alm_err(B16, B64) <= SPLIT_TOL


@pytest.mark.parametrize("ns,lmax,nsim", [(4, 11, 2), (16, 47, 5), (64, 191, 70), (512, 2048, 1)])
def test_split_eb2qu_matches_fp64(ns, lmax, nsim):
    """Spin-2 split synthesis (lambda1/lambda2 ring-row tiles, four passes with the factors
    -1, -i, +i and the south signs) against the plain path; lmax 2048 adds l-chunks."""
    rng = np.random.default_rng(ns)
    l = np.arange(lmax + 1, dtype=float)
    cl = np.where(l >= 2, 1.0 / np.maximum(l * (l + 1), 1.0), 0.0)
    E = gaussian_alm(cl, lmax, nsim, rng)
    B = gaussian_alm(0.1 * cl, lmax, nsim, rng)
    Q64, U64 = SHT(ns, lmax, nsim, pol=True).eb2qu(E, B)
    Q16, U16 = SHT(ns, lmax, nsim, pol=True, precision="split").eb2qu(E, B)
    assert rel_map_err(Q16, Q64) <= SPLIT_TOL
    assert rel_map_err(U16, U64) <= SPLIT_TOL


@pytest.mark.parametrize("ns,lmax", [(1, 0), (1, 2), (2, 1), (2, 5), (4, 0), (4, 16), (8, 32)])
def test_split_small_and_edge_sizes(ns, lmax):
    """Tiny rings, lmax 0 and lmax = 4 nside in every split transform (T and Q/U, both
    directions), against the plain path."""
    nsim = 3
    rng = np.random.default_rng(ns * 100 + lmax)
    maps = np.asfortranarray(rng.standard_normal((12 * ns * ns, nsim)))
    p64, p16 = SHT(ns, lmax, nsim, pol=True), SHT(ns, lmax, nsim, pol=True, precision="split")
    assert rel_alm_err(p16.t2alm(maps), p64.t2alm(maps)) <= SPLIT_TOL
    alm = p64.t2alm(maps)
    assert rel_map_err(p16.alm2t(alm), p64.alm2t(alm)) <= SPLIT_TOL
    if lmax >= 2:
        E64, B64 = p64.qu2eb(maps, maps[:, ::-1].copy(order="F"))
        E16, B16 = p16.qu2eb(maps, maps[:, ::-1].copy(order="F"))
        assert rel_alm_err(E16, E64) <= SPLIT_TOL and rel_alm_err(B16, B64) <= SPLIT_TOL
        Q64, U64 = p64.eb2qu(E64, B64)
        Q16, U16 = p16.eb2qu(E64, B64)
        assert rel_map_err(Q16, Q64) <= SPLIT_TOL and rel_map_err(U16, U64) <= SPLIT_TOL
