"""Plain FP64 parity with the oracle at the target sizes.

* nside 1024 / lmax 2047 (the precision-form configuration): at nside > 512 the reference
  seeds its recursion from tables (get_plm_recursive.f90:68-90) that this build and the
  oracle replace with an exponent-rescaled recursion, so this is where the two could part
  ways unnoticed.  t2alm (sht_main.f90:38-89) and alm2t (sht_main.f90:96-155), three maps.
* nside 256 / lmax 767 (the T + polarisation configuration): t2alm, alm2t, QU2EB
  (sht_main.f90:383-436) and EB2QU (sht_main.f90:1079-1147) on three I/Q/U sets drawn as
  that configuration draws them (C_l ~ 1/(l(l+1)) for l >= 2, E:B power 10:1, seed 1).

Bar: max_{l,m}|a - a_oracle| / max|a_oracle| <= 1e-11 per map (alm) and
max|T - T_oracle| / std(T_oracle) <= 1e-11 (maps), the plain method's bar.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import rel_alm_err, rel_map_err
from oracle import OracleSHT, gaussian_alm

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


def _cl(lmax, kind):
    l = np.arange(lmax + 1, dtype=float)
    if kind == "l-2":                       # C_l ~ l^-2, l >= 1 (a00 = 0)
        return np.where(l >= 1, 1.0 / np.maximum(l, 1.0) ** 2, 0.0)
    return np.where(l >= 2, 1.0 / np.maximum(l * (l + 1), 1.0), 0.0)   # 1/(l(l+1)), l >= 2


@pytest.fixture(scope="module")
def c3():
    ns, lmax, nsim = 1024, 2047, 3
    sht = SHT(ns, lmax, nsim)
    o = OracleSHT(ns, lmax, ring_tab=sht.ring_skip())
    rng = np.random.default_rng(2)
    alm = gaussian_alm(_cl(lmax, "l-2"), lmax, nsim, rng)
    return sht, o, alm


def test_alm2t_matches_oracle_at_nside_1024_lmax_2047(c3):
    sht, o, alm = c3
    got = sht.alm2t(alm)
    want = o.alm2t(alm)
    assert rel_map_err(got, want) <= TOL


def test_t2alm_matches_oracle_at_nside_1024_lmax_2047(c3):
    """Band-limited maps of the configuration's spectrum in the first two columns, white
    N(0, 1) pixels (power at every l up to the Nyquist ring) in the third."""
    sht, o, alm = c3
    maps = np.asfortranarray(sht.alm2t(alm))
    maps[:, 2] = np.random.default_rng(3).standard_normal(maps.shape[0])
    got = sht.t2alm(maps)
    want = o.t2alm(maps)
    assert rel_alm_err(got, want) <= TOL


@pytest.fixture(scope="module")
def c2():
    ns, lmax, nsim = 256, 767, 3
    sht = SHT(ns, lmax, nsim, pol=True)
    o = OracleSHT(ns, lmax, ring_tab=sht.ring_skip())
    rng = np.random.default_rng(1)
    cl = _cl(lmax, "l(l+1)")
    T = gaussian_alm(cl, lmax, nsim, rng)
    E = gaussian_alm(cl, lmax, nsim, rng)
    B = gaussian_alm(0.1 * cl, lmax, nsim, rng)
    return sht, o, T, E, B


def test_t_and_pol_synthesis_match_oracle_at_nside_256_lmax_767(c2):
    sht, o, T, E, B = c2
    assert rel_map_err(sht.alm2t(T), o.alm2t(T)) <= TOL
    Q, U = sht.eb2qu(E, B)
    Q0, U0 = o.eb2qu(E, B)
    assert rel_map_err(Q, Q0) <= TOL
    assert rel_map_err(U, U0) <= TOL


def test_t_and_pol_analysis_match_oracle_at_nside_256_lmax_767(c2):
    sht, o, T, E, B = c2
    I = np.asfortranarray(sht.alm2t(T))
    Q, U = (np.asfortranarray(x) for x in sht.eb2qu(E, B))
    assert rel_alm_err(sht.t2alm(I), o.t2alm(I)) <= TOL
    E1, B1 = sht.qu2eb(Q, U)
    E0, B0 = o.qu2eb(Q, U)
    assert rel_alm_err(E1, E0) <= TOL
    assert rel_alm_err(B1, B0) <= TOL
