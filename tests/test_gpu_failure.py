"""Failure detection without a GPU fault: every device-side wait of the
wavefront (the grid barrier between steps) is bounded.  A test hook makes the
barrier wait for an arrival that never comes; the wait runs out, the kernel
sets the context's error word and returns (no trap), wg_synchronize reports
WG_ERR_TIMEOUT, and after wg_clear_error and a restored state the same context
runs on and gives the bits of an undisturbed run."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_barrier_wait_runs_out_and_the_context_recovers():
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model, WgError
    region = sy.region_small_swb(seed=12)
    nd = 40
    P, T, S = sy.forcing(region, nd, doy0=90)
    q_ref = Model(region, max_days=nd).run(90, P, T, S)

    m = Model(region, max_days=nd)
    m.upload_forcing(0, P, T, S)
    m.save_snapshot()
    total = m.num_steps(nd)
    m.barrier_test(1)
    t0 = time.perf_counter()
    m.run_steps(90, 0, nd, 0, total)
    with pytest.raises(WgError, match="device wait exceeded its limit"):
        m.synchronize()
    assert time.perf_counter() - t0 < 60.0            # bounded: the waits ran out, nothing hung
    with pytest.raises(WgError):                       # results stay refused until the error is cleared
        m.discharge(0, nd)
    m.barrier_test(0)
    m.clear_error()
    m.restore_snapshot()
    m.run_steps(90, 0, nd, 0, total)
    assert np.array_equal(m.discharge(0, nd), q_ref)
