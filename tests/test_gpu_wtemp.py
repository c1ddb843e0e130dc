"""Water temperature on the GPU (wg_options.water_temp) against the oracle's
restatement of calcWaterTemp.cpp inside routing (itself pinned to the
reference: tests/test_wtemp_oracle.py), on the golden winter case with ice on
every kind of water body: the temperatures and ice thickness of every water
body, the stations' daily river temperature and the discharge."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-10   # |GPU - oracle| <= TOL * max(|oracle|, 1) (degC; km for ice against the 1e-9 floor below)


def _case():
    from watergap2_gb300.region import load_npz
    region, ex = load_npz(os.path.join(HERE, "golden", "swb_wtemp_90d.npz"))
    return region, ex


def _oracle(region, ex):
    from oracle import Oracle
    o = Oracle(region)
    o.init_water_temp(ex["GWT"])
    q, dt = o.run_wt(int(ex["doy0"]), ex["P"], ex["T"], ex["S"], ex["LW"], discharge=True, daily_temp=True)
    air = np.maximum(ex["T"].astype(np.float64), 0.0)
    return o, q, np.where(dt == -9999., air, dt)


def _model(region, ex, **kw):
    from watergap2_gb300.gpu import Model
    nd = ex["P"].shape[0]
    m = Model(region, max_days=nd, stations=ex["stations"], water_temp=True, **kw)
    m.set_water_temp_inputs(ex["GWT"], region.extras["river_length_file"])
    m.upload_forcing(0, ex["P"], ex["T"], ex["S"])
    m.upload_longwave(0, ex["LW"])
    return m


def _close(got, ref, floor):
    return np.abs(got - ref) <= TOL * np.maximum(np.abs(ref), floor)


def test_water_temperature_matches_oracle():
    region, ex = _case()
    nd, doy0 = ex["P"].shape[0], int(ex["doy0"])
    o, q_ref, t_ref = _oracle(region, ex)
    m = _model(region, ex)
    m.run_days(doy0, 0, nd)
    temp, ice = m.water_temp()
    assert _close(temp, o.wt["temp"], 1.0).all(), np.abs(temp - o.wt["temp"]).max()
    ok_ice = _close(ice, o.wt["ice"], 1e-9)
    assert ok_ice.all(), np.abs(ice - o.wt["ice"]).max()
    st = ex["stations"]
    assert _close(m.river_temp(0, nd), t_ref[:, st], 1.0).all()
    q = m.discharge(0, nd)
    assert np.all(np.abs(q - q_ref[:, st]) <= 1e-10 * np.maximum(np.abs(q_ref[:, st]), 1e-12))
    assert (ice > 0).any() and (temp[0] > 0).any()


def test_water_temperature_per_day_api_and_streaming():
    """The per-day entry points (the reference's call granularity) and a
    wavefront run split across calls give the same water temperatures."""
    region, ex = _case()
    nd, doy0 = ex["P"].shape[0], int(ex["doy0"])
    a = _model(region, ex)
    a.chunk_steps(7)
    total = a.num_steps(nd)
    for lo, hi in ((0, 11), (11, 60), (60, total)):
        a.run_steps(doy0, 0, nd, lo, hi)
    b = _model(region, ex)
    for d in range(nd):
        doy = (doy0 - 1 + d) % 365 + 1
        b.step_vertical(doy, d)
        b.step_routing(doy, d)
    ta, ia = a.water_temp()
    tb, ib = b.water_temp()
    assert _close(tb, ta, 1.0).all() and _close(ib, ia, 1e-9).all()
    ref = _model(region, ex)
    ref.run_days(doy0, 0, nd)
    tr, ir = ref.water_temp()
    assert np.array_equal(ta, tr) and np.array_equal(ia, ir)          # chunking changes no bit
    assert np.array_equal(a.river_temp(0, nd), ref.river_temp(0, nd))


def test_water_temperature_days_per_step():
    """Several days per wavefront step carry the river temperature through the
    same slots as the discharge: the same bits as one day per step."""
    region, ex = _case()
    nd, doy0 = ex["P"].shape[0], int(ex["doy0"])
    a = _model(region, ex)
    a.run_days(doy0, 0, nd)
    b = _model(region, ex, days_per_step=3)
    b.run_days(doy0, 0, nd)
    ta, ia = a.water_temp()
    tb, ib = b.water_temp()
    assert np.array_equal(ta, tb) and np.array_equal(ia, ib)
    assert np.array_equal(a.river_temp(0, nd), b.river_temp(0, nd))
    assert np.array_equal(a.discharge(0, nd), b.discharge(0, nd))
