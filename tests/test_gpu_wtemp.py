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


def test_global_grid_as_benchmarked_vs_oracle():
    """The global grid with fractional routing and the water temperature of
    every water body, in the bench's launch set-up (five days per wavefront
    step, chunks of four steps, the next chunk's vertical balance inside the
    wavefront launches), over a northern winter: the temperature and ice of
    every water body of every cell after 90 days, and the outlets' daily river
    temperature (within 1e-11 of the temperature in K) and discharge, against
    the oracle."""
    from oracle import Oracle
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_global().with_options(frac_routing=1)
    nd = 90
    P, T, S = sy.forcing(region, nd, seed=2, doy0=1)
    LW, GWT = sy.water_temp_inputs(region, nd, T)
    outlets = np.nonzero(region.downstream < 0)[0]
    m = Model(region, max_days=nd, stations=outlets, water_temp=True, days_per_step=5)
    assert m.vertical_overlap() > 0 and m.chunk_steps() == 4
    m.set_water_temp_inputs(GWT)
    m.upload_forcing(0, P, T, S)
    m.upload_longwave(0, LW)
    m.run_days(1, 0, nd)
    temp, ice = m.water_temp()
    tq, q = m.river_temp(0, nd), m.discharge(0, nd)
    del m
    o = Oracle(region)
    o.init_water_temp(GWT)
    q_ref, dt = o.run_wt(1, P, T, S, LW, discharge=True, daily_temp=True, nthreads=os.cpu_count() or 1)
    t_ref = np.where(dt == -9999., np.maximum(T.astype(np.float64), 0.0), dt)
    bad_t = ~_close(temp, o.wt["temp"], 1.0)
    bad_i = ~_close(ice, o.wt["ice"], 1e-9)
    print("global grid, 90 days: largest |temp diff|", np.abs(temp - o.wt["temp"]).max(),
          "largest |ice diff|", np.abs(ice - o.wt["ice"]).max(), "cells with ice", int((ice > 0).sum()))
    assert not bad_t.any(), np.argwhere(bad_t)[:5]
    assert not bad_i.any(), np.argwhere(bad_i)[:5]
    # a temperature is the energy over the heat capacity in K, less 273.15: its
    # rounding scales with the absolute temperature, and a river near 0 degC that
    # carries its upstream cells' rounding for weeks differs by ~1e-10 degC
    bad = np.argwhere(np.abs(tq - t_ref[:, outlets]) > 1e-11 * (np.abs(t_ref[:, outlets]) + 273.15))
    assert len(bad) == 0, (len(bad), [(int(d), int(outlets[j]), float(tq[d, j]), float(t_ref[d, outlets[j]]))
                                      for d, j in bad[:8]])
    assert np.all(np.abs(q - q_ref[:, outlets]) <= 1e-10 * np.maximum(np.abs(q_ref[:, outlets]), 1e-12))
    assert (ice > 0).sum() > 1000 and (ice[3:5] > 0).any()   # rivers and global lakes/reservoirs under ice
