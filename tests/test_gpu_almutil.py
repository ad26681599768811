"""alm utilities on the device (alm2cl, filt_alm, norm_alm, cl2alm) against the oracle's
restatements of the reference's Fortran, and the statistics of the Gaussian realisations."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import alm2cl as o_alm2cl, filt_alm as o_filt, norm_alm as o_norm, gaussian_alm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastsht_gb300 import build
    build.build()


def _alm(lmax, nsim, seed):
    rng = np.random.default_rng(seed)
    l = np.arange(lmax + 1, dtype=float)
    return gaussian_alm(1.0 / np.maximum(l, 1.0) ** 2, lmax, nsim, rng)


def test_alm2cl_matches_oracle_and_te_eb_order():
    from fastsht_gb300 import almutil
    lmax, nsim = 40, 5
    T, E, B = (_alm(lmax, nsim, s) for s in (1, 2, 3))
    cl = almutil.alm2cl(T, E, B, lmin=2)
    assert cl.shape == (nsim, lmax + 1, 6)
    want = [o_alm2cl(T, T, 2), o_alm2cl(E, E, 2), o_alm2cl(B, B, 2), o_alm2cl(T, E, 2),
            o_alm2cl(T, B, 2), o_alm2cl(E, B, 2)]
    for i, w in enumerate(want):
        assert np.abs(cl[..., i] - w).max() <= 1e-13 * np.abs(w).max()
    t = almutil.alm2cl(torch.from_numpy(np.ascontiguousarray(T.T)).cuda())   # library layout
    assert torch.is_tensor(t) and np.allclose(t.cpu().numpy(), o_alm2cl(T), rtol=1e-13)


def test_filt_and_norm_match_oracle():
    from fastsht_gb300 import almutil
    lmax, nsim = 33, 3
    a = _alm(lmax, nsim, 4)
    win = np.exp(-np.arange(lmax + 1) / 20.0)
    got = almutil.filt_alm(np.array(a, order="F", copy=True), win)
    assert np.abs(got - o_filt(a, win)).max() <= 1e-15
    shift = np.linspace(-1, 1, lmax + 1)
    got = almutil.norm_alm(a, win, shift, 2.5)
    assert np.abs(got - o_norm(a, win, shift, 2.5)).max() <= 1e-14


def test_cl2alm_statistics_and_reproducibility():
    """Realisations have the requested TT/EE/BB/TE spectra (ensemble mean within 5 sigma),
    zero below lmin, are identical for one seed and differ between seeds."""
    from fastsht_gb300 import almutil
    lmax, nsim, lmin = 24, 400, 2
    l = np.arange(lmax + 1, dtype=float)
    tt = np.where(l >= lmin, 1.0 / np.maximum(l * (l + 1), 1.0), 0.0)
    cl = np.stack([tt, 0.3 * tt, 0.05 * tt, 0.5 * np.sqrt(0.3) * tt, 0 * tt, 0 * tt], axis=1)
    T, E, B = almutil.cl2alm(cl, lmax, nsim, lmin=lmin, seed=11)
    T2, _, _ = almutil.cl2alm(cl, lmax, nsim, lmin=lmin, seed=11)
    T3, _, _ = almutil.cl2alm(cl, lmax, nsim, lmin=lmin, seed=12)
    assert torch.equal(T, T2) and not torch.equal(T, T3)
    spec = almutil.alm2cl(T, E, B)                      # (nsim, L, 6) tensor
    mean = spec.mean(dim=0).cpu().numpy()
    for i, col in enumerate([0, 1, 2, 3]):
        want = cl[:, col]
        for ll in range(lmin, lmax + 1):
            # C_l estimate of one map has variance ~2 C_l^2/(2l+1) (auto) or
            # (C_TT C_EE + C_TE^2)/(2l+1) (cross); mean over nsim maps
            var = (2 * want[ll] ** 2 if col < 3 else cl[ll, 0] * cl[ll, 1] + want[ll] ** 2) / (2 * ll + 1)
            assert abs(mean[ll, col] - want[ll]) <= 5 * np.sqrt(var / nsim), (col, ll)
    assert float(spec[:, :lmin, :].abs().max()) == 0.0
