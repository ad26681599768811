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
