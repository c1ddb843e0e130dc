"""wg_get_balance_noalloc, the balance sums for callers that cannot allocate
device memory once set up (one whose free device memory is held by another
framework's allocator, or one that sizes every buffer at start), against
wg_get_balance.

Collected last on purpose (file name), so that a failure here does not stop a
-x run before the other tests.  Runs alone in a fresh process as well as after
the other tests: the entry point's scratch address is looked up on its first
call on the device, whenever that is.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def test_noalloc_balance_matches_balance_on_two_calls():
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_small_swb(seed=17)
    P, T, S = sy.forcing(region, 120, doy0=60)
    m = Model(region, max_days=120, record_balance=True)
    m.upload_forcing(0, P, T, S)
    m.run_days(60, 0, 60)
    ref1, got1 = m.balance(), m.balance_noalloc()
    m.run_days(120, 60, 60)
    ref2, got2 = m.balance(), m.balance_noalloc()
    for ref, got in ((ref1, got1), (ref2, got2)):
        # storage, inflow, evaporation, outflow: compensated sums agree to 1e-12
        assert _rel(got[:4], ref[:4]) <= 1e-12, (got, ref)
        assert abs(got[4] - ref[4]) <= 1e-12 * max(abs(ref[1]), 1.0)
        assert got[5] == ref[5]          # largest residual: a max, order-independent
    assert not np.array_equal(got1, got2)   # the second call reports the later state


def test_noalloc_balance_fp32_ensemble():
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_small_swb(seed=18)
    P, T, S = sy.forcing(region, 40, doy0=200)
    m = Model(region, max_days=40, record_balance=True, precision="fp32", members=32,
              prec_factor=np.linspace(0.8, 1.2, 32).astype(np.float32))
    m.run(200, P, T, S)
    for _ in range(2):
        ref, got = m.balance(), m.balance_noalloc()
        assert _rel(got[:4], ref[:4]) <= 1e-12
        assert got[5] == ref[5]


def test_noalloc_balance_rejects_contexts_beyond_its_scratch():
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model, WgError
    region = sy.region_global()                    # 67,420 cells x 256 members > 16,777,216 states
    m = Model(region, max_days=2, record_balance=True, precision="fp32", members=256, ring_days=2)
    with pytest.raises(WgError, match="exceed its fixed scratch"):
        m.balance_noalloc()
    assert np.isfinite(m.balance()).all()          # the allocating entry point still works
