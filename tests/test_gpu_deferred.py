"""Deferred per-day calls (wg_set_deferred): the reference's day loop -- a
vertical-balance pass and a routing call per day, the model read at every month
end (integrateWGHM.cpp:767-860) -- queued and run as day-pipelined runs, with the
same bits as immediate per-day launches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MONTH_END = np.cumsum([31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31])


def _loop(m, doy0, nd, deferred, read_monthly=True):
    """Per-day calls; with read_monthly, the state and the month's discharge are
    read after the last day of every month."""
    if deferred:
        m.set_deferred(True)
    states = []
    for d in range(nd):
        doy = (doy0 - 1 + d) % 365 + 1
        m.step_vertical(doy, d)
        m.step_routing(doy, d)
        if read_monthly and doy in MONTH_END:
            states.append(m.get_state()["soil"].copy())
    q = m.discharge(0, nd)
    return q, m.get_state(), states


def test_deferred_days_equal_immediate_per_day_calls():
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_small_swb(seed=41)
    nd, doy0 = 200, 300
    P, T, S = sy.forcing(region, nd, doy0=doy0)
    runs = {}
    for name, deferred in (("immediate", False), ("deferred", True)):
        m = Model(region, max_days=nd, stations=np.arange(region.ncell))
        m.upload_forcing(0, P, T, S)
        l0 = m.launch_count
        runs[name] = _loop(m, doy0, nd, deferred) + (m.launch_count - l0,)
    qa, sa, ma, la = runs["immediate"]
    qb, sb, mb, lb = runs["deferred"]
    assert np.array_equal(qa, qb)
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    assert len(ma) == len(mb) and all(np.array_equal(x, y) for x, y in zip(ma, mb))
    assert lb < la / 4, (la, lb)   # the months ran as pipelined launches, not 2 launches a day


def test_deferred_global_grid_matches_pipelined_run():
    """The global grid over a year through the deferred per-day calls (the
    bench's drop-in route) equals one wg_run_days launch bit for bit."""
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_global()
    nd = 365
    P, T, S = sy.forcing(region, nd, doy0=1)
    a = Model(region, max_days=nd)
    a.upload_forcing(0, P, T, S)
    a.run_days(1, 0, nd)
    b = Model(region, max_days=nd)
    b.upload_forcing(0, P, T, S)
    qb, sb, _ = _loop(b, 1, nd, True)
    assert np.array_equal(a.discharge(0, nd), qb)
    for k, v in a.get_state().items():
        assert np.array_equal(v, sb[k]), k


def test_deferred_breaks_and_pending_vertical():
    """A queue broken by a jump of the output slot, an upload between days and a
    vertical call read before its routing call: the same bits as immediate calls."""
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_small_swb(seed=42)
    nd = 60
    P, T, S = sy.forcing(region, nd, doy0=100)
    out = []
    for deferred in (False, True):
        m = Model(region, max_days=nd + 10, stations=np.arange(region.ncell))
        m.upload_forcing(0, P[:30], T[:30], S[:30])
        if deferred:
            m.set_deferred(True)
        for d in range(20):
            m.step_vertical(100 + d, d)
            m.step_routing(100 + d, d + 5 if d >= 10 else d)   # output slots jump after day 10
        m.upload_forcing(30, P[30:], T[30:], S[30:])            # an upload runs the queue first
        for d in range(20, 40):
            m.step_vertical(100 + d, d)
            m.step_routing(100 + d, d + 5)
        m.step_vertical(140, 40)                                 # read before its routing call
        mid = m.get_state()
        m.step_routing(140, 45)
        out.append((m.discharge(0, nd + 10), mid, m.get_state()))
    (qa, ma, sa), (qb, mb, sb) = out
    assert np.array_equal(qa, qb)
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
        assert np.array_equal(ma[k], mb[k]), k
