"""Serving form, host-side logic that needs no GPU: request identity in the scheduler's
queues and the slot rule that keeps reserved slots for small jobs."""
from types import SimpleNamespace

import pytest

torch = pytest.importorskip("torch")

from fastsht_gb300.serve import Request, Server


def test_requests_of_equal_shape_are_distinct_in_queues():
    """Two requests with the same kind, sizes and precision (and equal input values) are two
    queue entries: removing one leaves the other (field-wise equality would compare their
    input tensors)."""
    a = Request("t2alm", 64, 128, 3, "fp64", [torch.zeros(3, 10)], 0.0)
    b = Request("t2alm", 64, 128, 3, "fp64", [torch.zeros(3, 10)], 0.0)
    q = [a, b]
    assert b in q and a != b
    q.remove(b)
    assert q == [a] and b not in q


@pytest.mark.parametrize("free,small,want", [
    ([0, 3, 5], True, 0),      # small jobs take a reserved (high-priority) slot first
    ([3, 5], True, 3),         # ... or any free one
    ([0, 1, 4], False, 4),     # large jobs never take a reserved slot
    ([0, 1], False, None),     # ... and wait when only reserved slots are free
])
def test_reserved_slots_take_only_small_jobs(free, small, want):
    srv = SimpleNamespace(_free_slots=list(free), reserved=2)
    assert Server._slot_for(srv, small) == want


def test_cost_model_counts_whole_map_tiles():
    """A job of fewer maps than a 64-map tile costs the whole tile's contraction (only its ring
    FFTs scale with the maps), so the duration cap never splits a request below one tile."""
    for prec in ("fp64", "split"):
        one = Server.cost_s("t2alm", 1024, 2047, prec, 1)
        tile = Server.cost_s("t2alm", 1024, 2047, prec, 64)
        two = Server.cost_s("t2alm", 1024, 2047, prec, 65)
        fft_per_map = (0.4e-3 if prec == "split" else 1.3e-3)
        assert tile - one == pytest.approx(63 * fft_per_map, rel=1e-9)
        leg_tile = 64 * 4.0 * 1024 * 2048 * 2049 / (80e12 if prec == "split" else 1e12)
        assert two - tile == pytest.approx(leg_tile + fft_per_map, rel=1e-9)   # a second tile
    # Q/U pairs cost four times the T contraction
    t = Server.cost_s("t2alm", 256, 512, "fp64", 64) - 64 * 1.3e-3 / 16
    qu = Server.cost_s("qu2eb", 256, 512, "fp64", 64) - 2 * 64 * 1.3e-3 / 16
    assert qu == pytest.approx(4 * t, rel=1e-9)
