"""Parity of the CUDA path (through the C ABI) with the FP64 oracle.

Bar for the plain FP64 method: max_{l,m}|a - a_oracle| / max|a_oracle| <= 1e-11 per
map (alm), and max|T - T_oracle| / std(T_oracle) <= 1e-11 (maps).
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import rel_alm_err, rel_map_err
from oracle import OracleSHT, gaussian_alm, alm_square_to_healpy

pytestmark = pytest.mark.gpu

TOL = 1e-11


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastsht_gb300 import build
    build.build()


def SHT(*a, **k):
    from fastsht_gb300 import SHT as _S
    return _S(*a, **k)


def maps_normal(ns, nsim, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal((12 * ns * ns, nsim)))


def alm_powerlaw(lmax, nsim, seed, lmin=0):
    rng = np.random.default_rng(seed)
    l = np.arange(lmax + 1, dtype=float)
    cl = 1.0 / np.maximum(l, 1.0) ** 2
    cl[:lmin] = 0
    return gaussian_alm(cl, lmax, nsim, rng)


T_CASES = [(1, 4, 3), (2, 5, 2), (2, 8, 1), (4, 11, 5), (4, 0, 2), (4, 1, 2), (8, 23, 7),
           (8, 32, 2), (16, 47, 3), (16, 16, 2), (32, 95, 4), (64, 191, 100)]


@pytest.mark.parametrize("ns,lmax,nsim", T_CASES)
def test_t2alm_matches_oracle(ns, lmax, nsim):
    sht = SHT(ns, lmax, nsim)
    o = OracleSHT(ns, lmax, ring_tab=sht.ring_skip())
    maps = maps_normal(ns, nsim, 10 + ns)
    got = sht.t2alm(maps)
    want = o.t2alm(maps)
    assert got.shape == want.shape
    assert rel_alm_err(got, want) <= TOL


@pytest.mark.parametrize("ns,lmax,nsim", T_CASES)
def test_alm2t_matches_oracle(ns, lmax, nsim):
    sht = SHT(ns, lmax, nsim)
    o = OracleSHT(ns, lmax, ring_tab=sht.ring_skip())
    alm = alm_powerlaw(lmax, nsim, 20 + ns)
    got = sht.alm2t(alm)
    want = o.alm2t(alm)
    assert got.shape == (12 * ns * ns, nsim)
    assert rel_map_err(got, want) <= TOL


@pytest.mark.parametrize("ns", [1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 1024])
def test_ring_skip_table_matches_reference(golden_skip, ns):
    ref = golden_skip[f"ns_{ns}"]
    lmax = min(4 * ns, len(ref) - 1)
    sht = SHT(ns, lmax, 1)
    assert np.array_equal(sht.ring_skip(), ref[:lmax + 1])


P_CASES = [(2, 8, 2), (4, 11, 3), (8, 23, 3), (8, 32, 1), (16, 47, 2), (32, 95, 3), (64, 191, 8)]


@pytest.mark.parametrize("ns,lmax,nsim", P_CASES)
def test_qu2eb_matches_oracle(ns, lmax, nsim):
    sht = SHT(ns, lmax, nsim, pol=True)
    o = OracleSHT(ns, lmax, ring_tab=sht.ring_skip())
    Q = maps_normal(ns, nsim, 30 + ns)
    U = maps_normal(ns, nsim, 40 + ns)
    E, B = sht.qu2eb(Q, U)
    E0, B0 = o.qu2eb(Q, U)
    assert rel_alm_err(E, E0) <= TOL
    assert rel_alm_err(B, B0) <= TOL
    assert rel_alm_err(sht.qu2e(Q, U), E0) <= TOL
    assert rel_alm_err(sht.qu2b(Q, U), B0) <= TOL


@pytest.mark.parametrize("ns,lmax,nsim", P_CASES)
def test_eb2qu_matches_oracle(ns, lmax, nsim):
    sht = SHT(ns, lmax, nsim, pol=True)
    o = OracleSHT(ns, lmax, ring_tab=sht.ring_skip())
    E = alm_powerlaw(lmax, nsim, 50 + ns, lmin=2)
    B = alm_powerlaw(lmax, nsim, 60 + ns, lmin=2)
    Q, U = sht.eb2qu(E, B)
    Q0, U0 = o.eb2qu(E, B)
    assert rel_map_err(Q, Q0) <= TOL
    assert rel_map_err(U, U0) <= TOL


@pytest.mark.parametrize("method", ["old", "new"])
@pytest.mark.parametrize("ns,lmax,nsim,niter", [(4, 11, 2, 1), (8, 23, 3, 3), (32, 95, 2, 2)])
def test_t2alm_iterations_match_oracle(ns, lmax, nsim, niter, method):
    sht = SHT(ns, lmax, nsim, niter=niter)
    o = OracleSHT(ns, lmax, ring_tab=sht.ring_skip())
    maps = maps_normal(ns, nsim, 70 + ns)
    got = sht.t2alm(maps, method=method)
    want = o.t2alm_iter_old(maps, niter) if method == "old" else o.t2alm_iter(maps, niter)
    assert rel_alm_err(got, want) <= TOL


@pytest.mark.parametrize("ns,lmax,nsim,niter", [(4, 11, 2, 1), (16, 47, 2, 2)])
def test_qu2eb_iterations_match_oracle(ns, lmax, nsim, niter):
    sht = SHT(ns, lmax, nsim, niter=niter, pol=True)
    o = OracleSHT(ns, lmax, ring_tab=sht.ring_skip())
    Q = maps_normal(ns, nsim, 80 + ns)
    U = maps_normal(ns, nsim, 90 + ns)
    E, B = sht.qu2eb(Q, U)
    E0, B0 = o.qu2eb_iter_old(Q, U, niter)
    assert rel_alm_err(E, E0) <= TOL
    assert rel_alm_err(B, B0) <= TOL


def test_chunked_workspace_gives_same_result():
    ns, lmax, nsim = 16, 47, 9
    maps = maps_normal(ns, nsim, 5)
    full = SHT(ns, lmax, nsim).t2alm(maps)
    per_map = (lmax + 1) * 2 * ns * 32
    small = SHT(ns, lmax, nsim, workspace_limit=2 * per_map + 1)
    assert small.plan_info()["maps_per_chunk"] == 2
    assert np.array_equal(small.t2alm(maps), full)
    alm = alm_powerlaw(lmax, nsim, 6)
    assert np.array_equal(small.alm2t(alm), SHT(ns, lmax, nsim).alm2t(alm))


def test_c1_config_roundtrip_and_healpy():
    """Config 1 shape: nside 64, lmax 191, 100 maps, N(0,1) seed 0; complex128
    healpy-ordered output through convert_alm_healpy."""
    ns, lmax, nsim = 64, 191, 100
    rng = np.random.default_rng(0)
    maps = np.asfortranarray(rng.standard_normal((12 * ns * ns, nsim)))
    sht = SHT(ns, lmax, nsim)
    o = OracleSHT(ns, lmax, ring_tab=sht.ring_skip())
    alm = sht.t2alm(maps)
    hp = sht.convert_alm_healpy(alm)
    assert hp.dtype == np.complex128 and hp.shape == ((lmax + 1) * (lmax + 2) // 2, nsim)
    want = alm_square_to_healpy(o.t2alm(maps))
    assert np.abs(hp - want).max() <= TOL * np.abs(want).max()
    back = sht.convert_alm_healpy_inv(hp)
    assert np.array_equal(back, alm)
    maps2 = sht.alm2t(alm)
    assert rel_map_err(maps2, o.alm2t(alm)) <= TOL


def test_torch_device_tensors_stay_on_device():
    ns, lmax, nsim = 8, 23, 3
    sht = SHT(ns, lmax, nsim)
    maps = maps_normal(ns, nsim, 3)
    dmaps = torch.from_numpy(maps.T.copy()).cuda().T          # (npix, nsim), Fortran strides
    dalm = sht.t2alm(dmaps)
    assert isinstance(dalm, torch.Tensor) and dalm.is_cuda and dalm.shape == (nsim, lmax + 1, lmax + 1)
    assert np.array_equal(dalm.cpu().numpy(), sht.t2alm(maps))
    back = sht.alm2t(dalm)
    assert back.is_cuda and back.shape == (12 * ns * ns, nsim)


def test_get_alm_false_then_get_alms():
    ns, lmax, nsim = 8, 23, 2
    sht = SHT(ns, lmax, nsim)
    maps = maps_normal(ns, nsim, 4)
    assert sht.t2alm(maps, get_alm=False) is None
    assert np.array_equal(sht.get_alms(), sht.t2alm(maps))
    out = np.empty((nsim, lmax + 1, lmax + 1), order="F")
    assert sht.t2alm(maps, alms_in=out) == 0
    assert np.array_equal(out, sht.get_alms())


def test_errors():
    sht = SHT(8, 23, 2)
    with pytest.raises(ValueError):
        sht.t2alm()                                 # no maps (SHT.py:78)
    with pytest.raises(ValueError):
        sht.t2alm(np.zeros((768, 3), order="F"))    # wrong nsim
    with pytest.raises(ValueError):
        sht.qu2eb(np.zeros((768, 2), order="F"), np.zeros((768, 2), order="F"))  # pol=False plan
    with pytest.raises(ValueError):
        SHT(3, 8, 1)                                # nside not a power of two


def test_linearity_at_c3_size():
    """nside 1024 / lmax 2047 (the precision-form config): t2alm is linear and
    alm2t(t2alm) reproduces a band-limited map's alm to the quadrature error."""
    ns, lmax, nsim = 1024, 2047, 2
    sht = SHT(ns, lmax, nsim)
    alm = alm_powerlaw(lmax, nsim, 2)
    alm[:, 0, 0] = 0
    m = sht.alm2t(alm)
    a1 = sht.t2alm(m)
    a2 = sht.t2alm(2.5 * m)
    assert rel_alm_err(a2, 2.5 * a1) <= 1e-13
    assert rel_alm_err(a1, alm) < 1e-2


def test_plans_of_different_sizes_coexist():
    """A later, smaller plan must not break an earlier plan's kernel launches."""
    big = SHT(64, 191, 2)
    maps = maps_normal(64, 2, 9)
    a1 = big.t2alm(maps)
    small = SHT(2, 5, 1)
    small.t2alm(maps_normal(2, 1, 1))
    assert np.array_equal(big.t2alm(maps), a1)
    assert big.alm2t(a1).shape == (12 * 64 * 64, 2)


def test_nside_2048_half_length_rings_match_oracle():
    """nside 2048: cap rings longer than 4096 pixels are transformed at half length (each
    ring's even/odd samples packed), forward and inverse; lmax 64 keeps the oracle quick."""
    ns, lmax, nsim = 2048, 64, 1
    sht = SHT(ns, lmax, nsim)
    o = OracleSHT(ns, lmax, ring_tab=sht.ring_skip())
    maps = maps_normal(ns, nsim, 2048)
    assert rel_alm_err(sht.t2alm(maps), o.t2alm(maps)) <= TOL
    alm = alm_powerlaw(lmax, nsim, 2049)
    assert rel_map_err(sht.alm2t(alm), o.alm2t(alm)) <= TOL


def test_nside_2048_lmax_4096_roundtrip_and_split():
    """The serving configuration's largest size, nside 2048 / lmax 4096: the split form
    against the plain path, and a synthesis -> analysis round trip of a band-limited map."""
    ns, lmax, nsim = 2048, 4096, 1
    alm = alm_powerlaw(lmax, nsim, 7, lmin=1)
    sht = SHT(ns, lmax, nsim)
    maps = sht.alm2t(alm)
    a64 = sht.t2alm(maps)
    a16 = SHT(ns, lmax, nsim, precision="split").t2alm(maps)
    assert rel_alm_err(a16, a64) <= 1e-7
    # niter = 0 quadrature error only (lmax = 2 nside): bounded, not exact
    assert rel_alm_err(a64, alm) < 0.5


@pytest.mark.parametrize("niter", [0, 2])
def test_fix_eb_matches_oracle(niter):
    """EB-leakage cleaning (SHT.fix_eb) against the oracle's restatement of fix_eb, and the
    reference's in-place masking of Q/U."""
    ns, lmax, nsim = 16, 40, 3
    rng = np.random.default_rng(5)
    l = np.arange(lmax + 1, dtype=float)
    cl = np.where(l >= 2, 1.0 / np.maximum(l * (l + 1), 1.0), 0.0)
    E = gaussian_alm(cl, lmax, nsim, rng)
    B = gaussian_alm(0.01 * cl, lmax, nsim, rng)
    sht = SHT(ns, lmax, nsim, niter=niter, pol=True)
    Q, U = sht.eb2qu(E, B)
    th = np.arccos(np.linspace(1, -1, 12 * ns * ns))           # a band mask, not healpy
    mask = (np.abs(np.cos(th)) > 0.3).astype(float)
    Qo, Uo = np.array(Q, order="F", copy=True), np.array(U, order="F", copy=True)
    want = OracleSHT(ns, lmax, ring_tab=sht.ring_skip()).fix_eb(Qo, Uo, mask, niter)
    got = sht.fix_eb(Q, U, mask)
    assert rel_map_err(got, want) <= 1e-10
    assert np.array_equal(Q, Qo * mask[:, None])               # masked in place
