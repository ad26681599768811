"""Failure detection on the device without a fault: a bounded wait that nothing satisfies
expires, raises the plan's error word, and the host sees FSHT_ETIMEOUT; the context stays
usable and the word is cleared."""
import ctypes as C

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


def test_expired_wait_is_reported_and_cleared():
    from fastsht_gb300 import SHT, _lib
    lib = _lib.load()
    sht = SHT(8, 23, 2, precision="split")
    assert lib.fsht_plan_sync(sht._plan) == _lib.FSHT_OK
    assert lib.fsht_selftest_wait_timeout(sht._plan) == _lib.FSHT_OK
    assert lib.fsht_plan_sync(sht._plan) == _lib.FSHT_ETIMEOUT
    assert "wait" in _lib.last_error()
    assert lib.fsht_plan_sync(sht._plan) == _lib.FSHT_OK          # cleared
    # the context is still usable: a transform afterwards is correct
    rng = np.random.default_rng(0)
    maps = np.asfortranarray(rng.standard_normal((12 * 64, 2)))
    a = sht.t2alm(maps)
    b = SHT(8, 23, 2).t2alm(maps)
    assert np.abs(a - b).max() <= 1e-7 * np.abs(b).max()


def test_non_finite_input_is_reported_by_the_split_form():
    """A NaN pixel cannot be cut into BF16 digits against any scale: the slicing kernel raises
    the plan's error word and the call fails with FSHT_ERANGE instead of returning alm whose
    digits were silently zeroed; the word is cleared and the next finite call is correct."""
    from fastsht_gb300 import SHT, _lib
    lib = _lib.load()
    rng = np.random.default_rng(1)
    maps = np.asfortranarray(rng.standard_normal((12 * 64, 2)))
    bad = maps.copy(order="F")
    bad[100, 1] = np.nan
    sht = SHT(8, 23, 2, precision="split")
    with pytest.raises(_lib.FshtError) as ei:
        sht.t2alm(torch.from_numpy(bad.T.copy()).cuda().T)
    assert ei.value.code == _lib.FSHT_ERANGE
    assert "digit scale" in str(ei.value)
    assert lib.fsht_plan_sync(sht._plan) == _lib.FSHT_OK          # cleared
    a = sht.t2alm(maps)
    b = SHT(8, 23, 2).t2alm(maps)
    assert np.abs(a - b).max() <= 1e-7 * np.abs(b).max()
