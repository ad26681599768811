"""Batched form: mixed map sets in one CUDA-graph launch give the same results as
the single-plan entry points, on the first (capturing) run and on graph replays."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import rel_alm_err
from oracle import gaussian_alm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fastsht_gb300 import build
    build.build()


def _alm(lmax, nmaps, seed):
    rng = np.random.default_rng(seed)
    l = np.arange(lmax + 1, dtype=float)
    cl = 1.0 / np.maximum(l, 1.0) ** 2
    cl[:2] = 0
    return gaussian_alm(cl, lmax, nmaps, rng)


def _dev_alm(a):           # (nsim, L, L) Fortran -> (L, L, nsim) contiguous device
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()


def test_mixed_batch_matches_single_plans():
    from fastsht_gb300 import SHT
    from fastsht_gb300.batch import Batch
    rng = np.random.default_rng(3)
    specs = [("t2alm", 8, 23, 3, "fp64"), ("qu2eb", 8, 20, 2, "fp64"),
             ("alm2t", 16, 40, 5, "fp64"), ("eb2qu", 16, 33, 2, "fp64"),
             ("t2alm", 32, 70, 7, "split"), ("t2alm", 32, 95, 1, "fp64"),
             ("qu2eb", 4, 11, 4, "fp64"), ("t2alm", 64, 150, 9, "split"),
             ("alm2t", 8, 23, 2, "fp64"), ("t2alm", 16, 40, 70, "split"),
             ("qu2eb", 32, 70, 3, "split"), ("alm2t", 32, 70, 4, "split")]
    b = Batch(nslots=3)
    refs = []
    for i, (kind, ns, lmax, nmaps, prec) in enumerate(specs):
        j = b.add(kind, ns, lmax, nmaps, precision=prec)
        sht = SHT(ns, lmax, nmaps, pol=kind in ("qu2eb", "eb2qu"), precision=prec)
        if kind in ("t2alm", "qu2eb"):
            maps = [sht.alm2t(_alm(lmax, nmaps, 10 * i + f)) for f in range(len(j.inputs))]
            for t, m in zip(j.inputs, maps):
                t.copy_(torch.from_numpy(np.ascontiguousarray(m.T)))
            if kind == "t2alm":
                refs.append([_dev_alm(sht.t2alm(maps[0]))])
            else:
                E, B = sht.qu2eb(maps[0], maps[1])
                refs.append([_dev_alm(E), _dev_alm(B)])
        else:
            alms = [_alm(lmax, nmaps, 10 * i + f) for f in range(len(j.inputs))]
            for t, a in zip(j.inputs, alms):
                t.copy_(_dev_alm(a))
            if kind == "alm2t":
                refs.append([torch.from_numpy(np.ascontiguousarray(sht.alm2t(alms[0]).T)).cuda()])
            else:
                Q, U = sht.eb2qu(alms[0], alms[1])
                refs.append([torch.from_numpy(np.ascontiguousarray(x.T)).cuda() for x in (Q, U)])
    b.build()
    for rep in range(3):
        for j in b.jobs:
            for t in j.outputs:
                t.fill_(float("nan"))
        b.run()
        b.sync()
        for j, ref in zip(b.jobs, refs):
            for got, want in zip(j.outputs, ref):
                assert torch.isfinite(got).all()
                scale = want.abs().max().item()
                err = (got - want).abs().max().item() / scale
                # split jobs: identical to the split single-plan path
                assert err <= 1e-12, (j.kind, j.nside, j.lmax, j.precision, rep, err)
    info = b.info()
    assert info["graph_nodes"] > 0 and info["plans"] == len({(s[1], s[2], s[4]) for s in specs})


def test_config4_style_batch_runs_and_is_deterministic():
    """Config-4 recipe, scaled down: nside log-uniform {32, 64, 128}, lmax uniform in
    [2 nside, 3 nside - 1], nmaps uniform 1..16, half T-only and half I/Q/U (seed 3)."""
    from fastsht_gb300.batch import Batch
    rng = np.random.default_rng(3)
    b = Batch(nslots=4)
    for s in range(12):
        ns = int(2 ** rng.integers(5, 8))
        lmax = int(rng.integers(2 * ns, 3 * ns))
        nmaps = int(rng.integers(1, 17))
        jT = b.add("t2alm", ns, lmax, nmaps)
        jT.inputs[0].normal_()
        if s % 2:
            jP = b.add("qu2eb", ns, lmax, nmaps)
            for t in jP.inputs:
                t.normal_()
    b.build()
    b.run()
    b.sync()
    first = [t.clone() for j in b.jobs for t in j.outputs]
    b.run()
    b.sync()
    again = [t for j in b.jobs for t in j.outputs]
    for x, y in zip(first, again):
        assert torch.equal(x, y)


def _rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    n = b.shape[0]
    return float((np.abs(a - b).reshape(n, -1).max(axis=1) /
                  np.abs(b).reshape(n, -1).max(axis=1)).max())


@pytest.mark.parametrize("mt,rc", [(32, 16), (64, 32), (32, 8), (64, 8)])
def test_fp64_contraction_shapes_give_the_same_transform(mt, rc):
    """Every FP64 analysis tile shape the autotuner may pick (maps per CTA, rings per chunk)
    gives the default shape's alm, T and Q/U, to FP64 rounding (the ring sums run in another
    order only when the rings per chunk change)."""
    import ctypes as C
    from fastsht_gb300 import SHT, _lib
    ns, lmax, nsim = 32, 80, 40
    rng = np.random.default_rng(mt + rc)
    T = np.asfortranarray(rng.standard_normal((12 * ns * ns, nsim)))
    Q = np.asfortranarray(rng.standard_normal((12 * ns * ns, nsim)))
    sht = SHT(ns, lmax, nsim, pol=True)
    a0 = sht.t2alm(T)
    e0, b0 = sht.qu2eb(Q, T)
    _lib.call("fsht_plan_set_contraction", sht._plan, mt, rc, 0)
    got = (C.c_int(), C.c_int(), C.c_int())
    _lib.call("fsht_plan_contraction", sht._plan, *[C.byref(x) for x in got])
    assert (got[0].value, got[1].value) == (mt, rc)
    assert _rel(sht.t2alm(T), a0) <= 1e-13
    e1, b1 = sht.qu2eb(Q, T)
    assert _rel(e1, e0) <= 1e-13 and _rel(b1, b0) <= 1e-13


@pytest.mark.parametrize("part", [16, 32])
def test_split_part_lengths_give_the_same_transform(part):
    """The split GEMMs' ring-part length (k-steps accumulated in TMEM before an FP64 add)
    changes only where the FP32 lower levels are rounded: T and E/B alm agree with the default
    64-step parts far inside the split form's 1e-7 bar."""
    from fastsht_gb300 import SHT, _lib
    ns, lmax, nsim = 512, 600, 9      # up to 1024 kept rings: 2 parts at 32 steps, 4 at 16
    rng = np.random.default_rng(part)
    T = np.asfortranarray(rng.standard_normal((12 * ns * ns, nsim)))
    Q = np.asfortranarray(rng.standard_normal((12 * ns * ns, nsim)))
    sht = SHT(ns, lmax, nsim, pol=True, precision="split")
    a0 = sht.t2alm(T)
    e0, b0 = sht.qu2eb(Q, T)
    _lib.call("fsht_plan_set_contraction", sht._plan, 0, 0, part)
    assert _rel(sht.t2alm(T), a0) <= 1e-9
    e1, b1 = sht.qu2eb(Q, T)
    assert _rel(e1, e0) <= 1e-9 and _rel(b1, b0) <= 1e-9


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_autotune_picks_a_contraction_shape(precision):
    """The autotuner times the FFT launch shapes and then the contraction's tile shapes, keeps
    one of the candidates and the transform stays the same."""
    import ctypes as C
    from fastsht_gb300 import SHT, _lib
    ns, lmax, nsim = 64, 160, 24
    rng = np.random.default_rng(7)
    T = np.asfortranarray(rng.standard_normal((12 * ns * ns, nsim)))
    sht = SHT(ns, lmax, nsim, precision=precision)
    a0 = sht.t2alm(T)
    _lib.call("fsht_plan_autotune", sht._plan, nsim)
    got = (C.c_int(), C.c_int(), C.c_int())
    _lib.call("fsht_plan_contraction", sht._plan, *[C.byref(x) for x in got])
    mt, rc, part = (x.value for x in got)
    if precision == "fp64":
        assert mt in (32, 64) and rc in (8, 16, 32) and part == 0
    else:
        assert part in (16, 32, 64) and mt == 0 and rc == 0
    tol = 1e-13 if precision == "fp64" else 1e-9
    assert _rel(sht.t2alm(T), a0) <= tol


def test_batch_reports_each_plans_tuned_shapes():
    """An autotuned batch of two buckets and both precisions reports one entry per plan with
    its key and shapes from the candidate sets, and its results equal an untuned batch's to
    each form's rounding."""
    from fastsht_gb300.batch import Batch
    outs = []
    for tune in (True, False):
        b = Batch(nslots=2, autotune=tune)
        for (ns, lmax, prec) in [(32, 80, "fp64"), (64, 160, "fp64"), (64, 160, "split")]:
            j = b.add("t2alm", ns, lmax, 12, precision=prec)
            g = torch.Generator(device=j.inputs[0].device)
            g.manual_seed(ns + lmax)
            j.inputs[0].copy_(torch.randn(j.inputs[0].shape, dtype=torch.float64,
                                          device=j.inputs[0].device, generator=g))
        b.build()
        b.run()
        b.sync()
        outs.append([t.cpu().numpy() for j in b.jobs for t in j.outputs])
        tun = b.tunings()
        b.close()
        assert len(tun) == 3
        keys = {(t["nside"], t["lmax"], t["precision"]) for t in tun}
        assert keys == {(32, 80, "fp64"), (64, 160, "fp64"), (64, 160, "split")}
        for t in tun:
            assert (1 <= t["fft_maps_per_cta"] <= 16) if tune else t["fft_maps_per_cta"] == 0
            if t["precision"] == "fp64":
                assert t["split_part_steps"] == 0
                if tune:
                    assert t["fp64_maps_per_cta"] in (32, 64)
                    assert t["fp64_rings_per_chunk"] in (8, 16, 32)
            else:
                assert t["fp64_maps_per_cta"] == 0 and t["fp64_rings_per_chunk"] == 0
                if tune:
                    assert t["split_part_steps"] in (16, 32, 64)
    for k, (x, y) in enumerate(zip(*outs)):
        tol = 1e-9 if k == 2 else 1e-13
        assert _rel(x[None], y[None]) <= tol
