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
