"""The oracle against the reference's golden vectors and analytic known answers
(CPU only)."""
import math

import numpy as np
import pytest
from scipy.special import sph_harm_y

from oracle import (OracleSHT, alm_healpy_to_square, alm_square_to_healpy, gaussian_alm,
                    plm_T, recursion_constants, ring_angles, ring_info, ring_skip_table)

from conftest import rel_alm_err, rel_map_err


@pytest.mark.parametrize("ns", [1, 2, 4, 8, 16, 32, 64, 128])
@pytest.mark.parametrize("scaled", [False, True])
def test_recursion_matches_plm_tables(golden_plm, ns, scaled):
    """lambda_{pos,m}, lambda_{pos+1,m} at the ring colatitudes against the
    reference's plm_table/*.bin (pins theta_i and the recursion)."""
    cols = golden_plm[f"cols_{ns}"]
    pos = golden_plm[f"pos_{ns}"]
    v1 = golden_plm[f"val1_{ns}"]
    v2 = golden_plm[f"val2_{ns}"]
    lmax = int(pos.max()) + 2
    th, _ = ring_angles(ns)
    k = recursion_constants(ns, lmax, th)
    worst = 0.0
    rows = np.arange(2 * ns)
    for j, m in enumerate(cols):
        lam = plm_T(int(m), lmax, ns, k, 0, scaled=scaled)
        for got, want in ((lam[rows, pos[:, j]], v1[:, j]), (lam[rows, pos[:, j] + 1], v2[:, j])):
            ok = np.abs(want) > (1e-250 if not scaled else 1e-80)
            if ok.any():
                worst = max(worst, float((np.abs(got[ok] - want[ok]) / np.abs(want[ok])).max()))
    assert worst < 1e-12, worst


@pytest.mark.parametrize("ns", [1, 2, 4, 8, 16, 32, 64])
def test_ring_skip_rule_matches_tables(golden_skip, ns):
    ref = golden_skip[f"ns_{ns}"]
    mine = ring_skip_table(ns, len(ref) - 1)
    assert np.array_equal(ref, mine)


def test_ring_geometry():
    for ns in (1, 2, 4, 16):
        i1, nfft = ring_info(ns)
        assert i1[0] == 0 and i1[-1] + nfft[-1] == 12 * ns * ns
        assert np.all(i1[1:] == i1[:-1] + nfft[:-1])
        assert np.array_equal(nfft, nfft[::-1])


def _pixel_angles(ns):
    i1, nfft = ring_info(ns)
    thn, ph0 = ring_angles(ns)
    th = np.concatenate([thn, math.pi - thn[:-1][::-1]])
    phi0 = np.concatenate([ph0, ph0[:-1][::-1]])
    T = np.empty(12 * ns * ns)
    P = np.empty(12 * ns * ns)
    for i in range(4 * ns - 1):
        j = np.arange(nfft[i])
        T[i1[i]:i1[i] + nfft[i]] = th[i]
        P[i1[i]:i1[i] + nfft[i]] = phi0[i] + 2 * math.pi * j / nfft[i]
    return T, P


def test_constant_map_a00():
    ns, lmax = 8, 23
    o = OracleSHT(ns, lmax)
    c = 1.7
    alm = o.t2alm(np.full((12 * ns * ns, 2), c, order="F"))
    assert abs(alm[0, 0, 0] - math.sqrt(4 * math.pi) * c) < 1e-12


@pytest.mark.parametrize("lm", [(0, 0), (1, 0), (1, 1), (5, 3), (10, 7), (23, 23), (20, 0)])
def test_synthesis_of_single_alm_is_ylm(lm):
    l, m = lm
    ns, lmax = 8, 23
    o = OracleSHT(ns, lmax)
    T, P = _pixel_angles(ns)
    a = np.zeros((1, lmax + 1, lmax + 1), order="F")
    a[0, l, m] = 0.3
    if m > 0:
        a[0, l - m, lmax + 1 - m] = -0.2
    mp = o.alm2t(a)[:, 0]
    ac = complex(0.3, -0.2) if m > 0 else 0.3
    want = (ac * sph_harm_y(l, m, T, P)).real * (2 if m > 0 else 1)
    assert np.abs(mp - want).max() < 1e-13


def test_iterations_reduce_roundtrip_error():
    ns, lmax = 8, 23
    o = OracleSHT(ns, lmax)
    rng = np.random.default_rng(0)
    alm = gaussian_alm(1.0 / (np.arange(lmax + 1) + 1.0) ** 2, lmax, 3, rng)
    mp = o.alm2t(alm)
    e0 = rel_alm_err(o.t2alm(mp), alm)
    e3 = rel_alm_err(o.t2alm_iter_old(mp, 3), alm)
    e3n = rel_alm_err(o.t2alm_iter(mp, 3), alm)
    assert e3 < e0 and e3n < e0


def test_spin2_roundtrip_and_parts():
    ns, lmax = 8, 2 * 8
    o = OracleSHT(ns, lmax)
    rng = np.random.default_rng(1)
    cl = np.zeros(lmax + 1)
    cl[2:] = 1.0 / (np.arange(2, lmax + 1) * np.arange(3, lmax + 2))
    E = gaussian_alm(cl, lmax, 2, rng)
    B = gaussian_alm(0.1 * cl, lmax, 2, rng)
    for a in (E, B):
        a[:, 1, 1] = 0
        a[:, 0, lmax] = 0
    Q, U = o.eb2qu(E, B)
    E1, B1 = o.qu2eb(Q, U)
    assert rel_alm_err(E1, E) < 0.05 and rel_alm_err(B1, B) < 0.3
    E3, B3 = o.qu2eb_iter_old(Q, U, 4)
    assert rel_alm_err(E3, E) < rel_alm_err(E1, E)
    assert np.array_equal(o.qu2e(Q, U), E1)
    assert np.abs(o.qu2b(Q, U) - B1).max() < 1e-14


def test_healpy_conversion_roundtrip():
    lmax = 9
    rng = np.random.default_rng(2)
    a = gaussian_alm(np.ones(lmax + 1), lmax, 3, rng)
    hp = alm_square_to_healpy(a)
    assert hp.shape == ((lmax + 1) * (lmax + 2) // 2, 3)
    # index m(2 lmax + 1 - m)/2 + l
    l, m = 7, 3
    idx = m * (2 * lmax + 1 - m) // 2 + l
    assert hp[idx, 1] == complex(a[1, l, m], a[1, l - m, lmax + 1 - m])
    assert np.array_equal(alm_healpy_to_square(hp, lmax), a)


@pytest.mark.slow
def test_scaled_and_unscaled_recursion_agree_on_kept_rings():
    """For nside <= 512 the reference seeds lambda_mm directly; the GPU uses the
    exponent-rescaled recursion.  On the rings the reference keeps they agree."""
    ns, lmax = 64, 191
    th, _ = ring_angles(ns)
    k = recursion_constants(ns, lmax, th)
    skip = ring_skip_table(ns, lmax)
    for m in range(0, lmax + 1, 7):
        a = plm_T(m, lmax, ns, k, int(skip[m]), scaled=False)
        b = plm_T(m, lmax, ns, k, int(skip[m]), scaled=True)
        assert np.abs(a - b).max() <= 1e-12 * max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("ns,lmax,scaled", [(8, 23, False), (8, 32, True), (64, 191, False),
                                             (64, 191, True)])
def test_c_recursion_matches_numpy(ns, lmax, scaled):
    from oracle import plm_c, plm_pol
    th, _ = ring_angles(ns)
    k = recursion_constants(ns, lmax, th)
    for m in (0, 1, 2, 5, lmax // 2, lmax):
        i0 = 0
        a = plm_T(m, lmax, ns, k, i0, scaled=scaled)
        p0, p1, p2 = plm_c(m, lmax, ns, k, i0, True, scaled=scaled)
        q1, q2 = plm_pol(m, lmax, ns, k, i0, a)
        sc = max(np.abs(a).max(), 1e-300)
        assert np.abs(p0 - a).max() <= 1e-13 * sc
        assert np.abs(p1 - q1).max() <= 1e-12 * max(np.abs(q1).max(), 1e-300)
        assert np.abs(p2 - q2).max() <= 1e-12 * max(np.abs(q2).max(), 1e-300)


def test_oracle_c_and_numpy_paths_agree():
    ns, lmax = 8, 23
    rng = np.random.default_rng(3)
    maps = np.asfortranarray(rng.standard_normal((12 * ns * ns, 2)))
    a = OracleSHT(ns, lmax, use_c=True).t2alm(maps)
    b = OracleSHT(ns, lmax, use_c=False).t2alm(maps)
    assert rel_alm_err(a, b) < 1e-13
    Q = np.asfortranarray(rng.standard_normal((12 * ns * ns, 2)))
    e1, b1 = OracleSHT(ns, lmax, use_c=True).qu2eb(Q, maps)
    e2, b2 = OracleSHT(ns, lmax, use_c=False).qu2eb(Q, maps)
    assert rel_alm_err(e1, e2) < 1e-13 and rel_alm_err(b1, b2) < 1e-13


def test_alm2cl_of_one_mode_and_linearity():
    """alm2cl restatement: a single Re a_lm = 1 at m > 0 gives C_l = 2/(2l+1); the m = 0
    mode gives 1/(2l+1); cross spectra are bilinear."""
    from oracle import alm2cl
    L = 9
    a = np.zeros((1, L, L), order="F")
    a[0, 5, 3] = 1.0                       # Re a_{5,3}
    cl = alm2cl(a)
    assert np.allclose(cl[0], np.where(np.arange(L) == 5, 2.0 / 11, 0.0))
    b = np.zeros((1, L, L), order="F")
    b[0, 4, 0] = 3.0                       # a_{4,0}
    assert np.isclose(alm2cl(b)[0, 4], 9.0 / 9)
    rng = np.random.default_rng(0)
    x = np.asfortranarray(rng.standard_normal((2, L, L)))
    y = np.asfortranarray(rng.standard_normal((2, L, L)))
    assert np.allclose(alm2cl(x + y), alm2cl(x) + 2 * alm2cl(x, y) + alm2cl(y))
    assert np.allclose(alm2cl(x, lmin=4)[:, :4], 0.0)


def test_filt_and_norm_restatements():
    from oracle import filt_alm, norm_alm
    L = 7
    rng = np.random.default_rng(1)
    a = np.asfortranarray(rng.standard_normal((3, L, L)))
    win = np.linspace(0.5, 1.5, L)
    f = filt_alm(a, win)
    assert np.isclose(f[1, 5, 2], a[1, 5, 2] * win[5])            # Re a_{5,2}
    assert np.isclose(f[1, 5 - 2, L - 2], a[1, 5 - 2, L - 2] * win[5])   # Im a_{5,2}
    n = norm_alm(a, win, np.full(L, 0.25), 3.0)
    assert np.isclose(n[0, 4, 0], a[0, 4, 0] * win[4] * 3.0 + 0.25)
    assert np.isclose(n[0, 4, 1], a[0, 4, 1] * win[4] + 0.25)


@pytest.mark.parametrize("ns,lmax,m", [(8, 23, 0), (8, 23, 5), (16, 47, 30), (32, 95, 95)])
def test_c_gather_matches_numpy_fft2mat(ns, lmax, m):
    """The C gather the CPU baseline times (reference memory order, map index fastest)
    forms the same FFT matrix as the NumPy restatement of fft2mat_fast."""
    o = OracleSHT(ns, lmax)
    rng = np.random.default_rng(m)
    maps = np.asfortranarray(rng.standard_normal((12 * ns * ns, 5)))
    buff = o.map2fft(maps)                          # (nsim, npix)
    m1, m2 = o.fft2mat(buff, m)                     # (nsim, rlen)
    c1, c2 = o.fft2mat_c(np.ascontiguousarray(buff.T), m)
    assert np.array_equal(c1, m1.T) and np.array_equal(c2, m2.T)
