"""Serving form: continuous batching with HBM-budget admission.  Each result is
the same alone and in a mix; requests overlap on the device; a request larger
than the budget is split along maps and still exact; the budget is respected."""
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


def _inputs(kind, ns, lmax, nmaps, gen):
    nf = 2 if kind in ("qu2eb", "eb2qu") else 1
    if kind in ("t2alm", "qu2eb"):
        return [torch.randn((nmaps, 12 * ns * ns), dtype=torch.float64, device="cuda",
                            generator=gen) for _ in range(nf)]
    L = lmax + 1
    return [torch.randn((L, L, nmaps), dtype=torch.float64, device="cuda", generator=gen)
            for _ in range(nf)]


def _direct(kind, ns, lmax, ins, precision):
    from fastsht_gb300 import SHT
    nmaps = ins[0].shape[0] if kind in ("t2alm", "qu2eb") else ins[0].shape[-1]
    sht = SHT(ns, lmax, nmaps, pol=kind in ("qu2eb", "eb2qu"), precision=precision)
    if kind == "t2alm":
        out = [sht.t2alm(ins[0].T)]
    elif kind == "alm2t":
        out = [sht.alm2t(ins[0].permute(2, 1, 0))]
    elif kind == "qu2eb":
        out = list(sht.qu2eb(ins[0].T, ins[1].T))
    else:
        out = list(sht.eb2qu(ins[0].permute(2, 1, 0), ins[1].permute(2, 1, 0)))
    # back to the library layouts
    if kind in ("t2alm", "qu2eb"):
        return [o.permute(2, 1, 0).contiguous() for o in out]
    return [o.T.contiguous() for o in out]


def _close(a, b, tol=1e-12):
    return (a - b).abs().max().item() <= tol * max(b.abs().max().item(), 1e-300)


def test_result_is_the_same_alone_and_in_a_mix():
    from fastsht_gb300.serve import Server
    gen = torch.Generator(device="cuda").manual_seed(4)
    probe = ("t2alm", 32, 80, 5, "split")
    pins = _inputs(*probe[:4], gen)
    torch.cuda.synchronize()
    srv = Server(hbm_budget=4e9, nslots=4)
    alone = srv.submit(probe[0], probe[1], probe[2], pins, precision=probe[4]).result(timeout=120)
    rng = np.random.default_rng(4)
    reqs = []
    for i in range(14):
        kind = ["t2alm", "alm2t", "qu2eb", "eb2qu"][i % 4]
        ns = int(2 ** rng.integers(3, 7))
        lmax = 2 * ns
        nmaps = int(rng.integers(1, 9))
        prec = "split" if (kind == "t2alm" and i % 3 == 0) else "fp64"
        ins = _inputs(kind, ns, lmax, nmaps, gen)
        reqs.append((kind, ns, lmax, ins, prec))
    torch.cuda.synchronize()
    futs = []
    for i, (kind, ns, lmax, ins, prec) in enumerate(reqs):
        futs.append(srv.submit(kind, ns, lmax, ins, precision=prec))
        if i == 6:
            mixed = srv.submit(probe[0], probe[1], probe[2], pins, precision=probe[4])
    srv.drain(timeout=300)
    st = srv.stats()
    assert st["max_inflight"] >= 2            # requests overlapped on the device
    for a, b in zip(mixed.result(), alone):
        assert torch.equal(a, b)
    for f, (kind, ns, lmax, ins, prec) in zip(futs, reqs):
        for got, want in zip(f.result(), _direct(kind, ns, lmax, ins, prec)):
            assert _close(got, want)
    assert st["p99_ms"] >= st["p50_ms"] > 0
    srv.close()


def test_request_larger_than_budget_is_split_and_exact():
    from fastsht_gb300.serve import Server
    gen = torch.Generator(device="cuda").manual_seed(5)
    ns, lmax, nmaps = 32, 64, 24
    ins = _inputs("t2alm", ns, lmax, nmaps, gen)
    torch.cuda.synchronize()
    budget = 2_500_000           # a few maps' worth
    srv = Server(hbm_budget=budget, nslots=3)
    out = srv.submit("t2alm", ns, lmax, ins).result(timeout=120)
    srv.drain()
    st = srv.stats()
    assert st["high_water_bytes"] <= budget
    assert srv.completed[0].parts > 1
    assert _close(out[0], _direct("t2alm", ns, lmax, ins, "fp64")[0])
    srv.close()


def test_waiting_requests_of_one_configuration_are_fused():
    """Requests of one (kind, nside, lmax, precision) that wait together run as one job
    along the map axis; each still gets its own maps' results."""
    from fastsht_gb300.serve import Server
    gen = torch.Generator(device="cuda").manual_seed(6)
    ns, lmax = 64, 128
    blocker = _inputs("t2alm", 256, 512, 16, gen)        # keeps the single slot busy
    reqs = [_inputs("t2alm", ns, lmax, n, gen) for n in (3, 1, 5, 2)]
    torch.cuda.synchronize()
    srv = Server(hbm_budget=8e9, nslots=1)
    srv.submit("t2alm", 256, 512, blocker)
    futs = [srv.submit("t2alm", ns, lmax, ins) for ins in reqs]
    srv.drain(timeout=120)
    assert srv.stats()["max_fused"] >= 2
    for f, ins in zip(futs, reqs):
        got = f.result()[0]
        want = _direct("t2alm", ns, lmax, ins, "fp64")[0]
        assert got.shape == want.shape and _close(got, want)
    srv.close()


def test_small_requests_are_not_held_behind_a_large_one():
    """Head-of-line blocking: an FP64 request of 256 maps at nside 1024 (several seconds of GPU
    time) is in flight when small requests arrive.  It runs as several jobs of one 64-map tile
    (the max_job_s cap, never below a tile), and the small ones run on the reserved
    high-priority slots, whose thread blocks the scheduler starts ahead of the large job's
    waiting blocks.  Thread blocks are not preempted, so a small request can still wait for
    large-job blocks already running (an FP64 analysis block of a 64-map tile at nside 1024
    runs for a few tenths of a second, and a small job has several kernels), but not for the
    large request: every small one finishes in well under the large one's time, most of them
    in a small fraction of it, with its result unchanged."""
    import time
    from fastsht_gb300.serve import Server
    gen = torch.Generator(device="cuda").manual_seed(11)
    big = _inputs("t2alm", 1024, 2047, 256, gen)
    small = [_inputs("t2alm", 32, 64, 1, gen) for _ in range(6)]
    torch.cuda.synchronize()
    srv = Server(hbm_budget=60e9, nslots=4, max_job_s=0.25)
    try:
        # plans and kernels of both configurations in place first
        srv.submit("t2alm", 1024, 2047, [big[0][:1].contiguous()], "fp64").result(timeout=300)
        srv.submit("t2alm", 32, 64, small[0], "fp64").result(timeout=60)
        srv.drain()
        srv.completed.clear()
        fb = srv.submit("t2alm", 1024, 2047, big, "fp64")
        time.sleep(0.05)
        fs = [srv.submit("t2alm", 32, 64, s, "fp64") for s in small]
        outs = [f.result(timeout=300) for f in fs]
        fb.result(timeout=600)
        st = srv.stats()
        lat = {}
        for r in srv.completed:
            lat.setdefault(r.nside, []).append(r.t_done - r.t_arrival)
        big_req = [r for r in srv.completed if r.nside == 1024][0]
    finally:
        srv.close()
    assert big_req.parts >= 4, big_req.parts                 # ran as several capped jobs
    big_t = lat[1024][0]
    assert max(lat[32]) < 0.6 * big_t, (lat, st)             # not held behind the request
    assert float(np.median(lat[32])) < 0.3 * big_t, (lat, st)
    want = _direct("t2alm", 32, 64, small[3], "fp64")
    assert _close(outs[3][0], want[0])


def test_budget_holds_outputs_until_completion_and_is_released():
    """A request split into several jobs keeps every finished piece's output charged until it
    completes; afterwards nothing stays charged, the high-water mark respects the budget, and a
    discarding server completes futures with None."""
    from fastsht_gb300.serve import Server
    gen = torch.Generator(device="cuda").manual_seed(9)
    ns, lmax = 32, 64
    big = _inputs("t2alm", ns, lmax, 24, gen)
    small = [_inputs("alm2t", ns, lmax, 3, gen) for _ in range(3)]
    torch.cuda.synchronize()
    budget = 3_000_000
    for discard in (False, True):
        srv = Server(hbm_budget=budget, nslots=3, discard_outputs=discard)
        try:
            fb = srv.submit("t2alm", ns, lmax, big)
            fs = [srv.submit("alm2t", ns, lmax, x) for x in small]
            out = fb.result(timeout=120)
            outs = [f.result(timeout=120) for f in fs]
            srv.drain()
            st = srv.stats()
            assert st["high_water_bytes"] <= budget
            assert max(r.parts for r in srv.completed) > 1
            assert srv._used == 0
            if discard:
                assert out is None and all(o is None for o in outs)
            else:
                assert _close(out[0], _direct("t2alm", ns, lmax, big, "fp64")[0])
                assert _close(outs[1][0], _direct("alm2t", ns, lmax, small[1], "fp64")[0])
        finally:
            srv.close()
