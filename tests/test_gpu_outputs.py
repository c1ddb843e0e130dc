"""Monthly and daily output grids on the GPU against the reference's own grids.

The fixture swb_outputs_730d holds the reference's grids (options grid_store = 6,
storages at the month's end, outMinMaxRiverAvail = 1, the daily output options
on) of the second of two calendar years on a 281-cell region with every
water-body type and inland sinks: the vertical balance's 29 monthly sums and
means (daily.cpp:1281-1386) with total PET (1303) and its canopy, snow and soil
storages at the month's end; routing's river availability with its minimum and
maximum, cell runoff and velocity (routing.cpp:3964-4040) and every routing
storage at the month's end (routing.cpp:4725-4737) and routing's further grids
(open-water evaporation, cell surface runoff, groundwater runoff, land-area
fraction, wetland extents, reservoir inflow and outflow, consistent
precipitation, surface storage, cell AET); and the daily grids of both
(daily.cpp:1388-1399, 1472-1540; routing.cpp:4113-4210, 4620-4634) on a sample
of days.

Tolerance (FP64): 1e-10 relative to each grid's values, elements below 1e-6 of
the grid's largest value compared against that floor (helpers.max_rel_err).
"""
import os

import numpy as np
import pytest

from helpers import max_rel_err

pytestmark = pytest.mark.gpu
RTOL = 1e-10
PATH = os.path.join(os.path.dirname(__file__), "golden", "swb_outputs_730d.npz")
# the same grids with water use met in the cell (subtract_use = 2)
PATH_WU = os.path.join(os.path.dirname(__file__), "golden", "swb_outputs_wuse_730d.npz")
# and with the riparian cells' NUs met by their outflow cell (GLWD units)
PATH_GL = os.path.join(os.path.dirname(__file__), "golden", "swb_outputs_glwd_730d.npz")
Y2 = 365   # the grids are the second year's
# with water use, routing's flux grids against a floor of 1 % of each grid's largest value
RTOL_WU = 1e-7
FLUX_WU = ["river_avail", "min_avail", "max_avail", "cell_runoff", "velocity", "cell_surface_runoff",
           "open_water_evap", "cell_aet", "cell_aet_wca", "res_inflow", "res_outflow", "actual_use", "nug",
           "consistent_precip", "surf_storage", "gw_runoff",
           "d_r_river_avail", "d_r_velocity", "d_r_cell_runoff", "d_r_cell_runoff_mm", "d_r_cell_surface_runoff",
           "d_r_gw_runoff", "d_r_cell_aet", "d_r_consistent_precip"]
# Model.monthly name -> the reference's grid
ROUTING = {"river_avail": "river_avail", "min_avail": "min_river_avail", "max_avail": "max_river_avail",
           "cell_runoff": "cell_runoff", "velocity": "velocity"}
# rows of Model.daily_storages
STORAGES = ["loclake", "locwetl", "glolake", "glowetl", "res", "river", "gw"]
MONTH_END = np.cumsum([31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31]) - 1


@pytest.fixture(scope="module", autouse=True)
def _built():
    from watergap2_gb300 import build, gpu
    if not os.path.exists(gpu.LIB_PATH):
        build.build()


def _two_years(days_per_step=0, deferred=False, routing=True, wuse=False):
    from watergap2_gb300.gpu import Model
    from watergap2_gb300.region import load_npz
    region, ex = load_npz({False: PATH, True: PATH_WU, "glwd": PATH_GL}[wuse])
    P, T, S = ex["P"], ex["T"], ex["S"]
    nd = P.shape[0]
    kw = {"glwd_unit": ex["GLWD"]} if wuse == "glwd" else {}
    m = Model(region, max_days=nd, stations=ex["stations"], days_per_step=days_per_step, water_use=bool(wuse), **kw)
    if wuse:
        m.set_water_use_inputs(ex["FRGI"])
        m.upload_water_use_run(0, 1, nd, (ex["NUS"], ex["NUG"], ex["WDR"], ex["CONS"]))
    m.monthly_outputs(24, doy_day0=1)
    m.monthly_outputs_vertical(True)
    m.daily_outputs_vertical(nd)
    if routing:
        m.monthly_outputs_routing(True)
        m.daily_outputs_routing(nd)
    m.record_daily_storages(True)
    m.upload_forcing(0, P, T, S)
    if deferred:                                       # per-day calls, queued into day-pipelined runs
        m.set_deferred(True)
        for d in range(nd):
            doy = d % 365 + 1
            m.step_vertical(doy, d)
            m.step_routing(doy, d)
    else:
        m.run_days(1, 0, nd)
    grids = {k: m.monthly(k, 12, 12) for k in m.MONTHLY_VERTICAL + list(ROUTING)}
    grids.update({"d_" + k: m.daily_vertical(k, Y2, 365) for k in m.DAILY_VERTICAL})
    if routing:
        grids.update({k: m.monthly(k, 12, 12) for k in m.MONTHLY_ROUTING + ["cell_aet", "cell_aet_wca"]})
        grids.update({"d_r_" + k: m.daily_routing(k, Y2, 365) for k in m.DAILY_ROUTING})
    return m, ex, grids


@pytest.mark.parametrize("dps,routing,wuse", [(1, True, False), (5, True, False), (5, False, False),
                                              (1, True, True), (5, True, True), (5, True, "glwd")])
def test_output_grids_match_reference(dps, routing, wuse):
    """All grids (routing's further grids with the vertical balance's: the
    wavefront's variant with both), the vertical balance's grids alone (its
    variant without routing's further terms), and all grids with water use."""
    m, ex, grids = _two_years(days_per_step=dps, routing=routing, wuse=wuse)
    errs = {k: max_rel_err(grids[k], ex["m_" + k]) for k in m.MONTHLY_VERTICAL}
    errs.update({k: max_rel_err(grids[k], ex["m_" + r]) for k, r in ROUTING.items()})
    ds = m.daily_storages(Y2, 365)
    for i, f in enumerate(STORAGES):
        errs[f + "_storage"] = max_rel_err(ds[MONTH_END, i], ex[f"m_{f}_storage"])
        if wuse and f == "river":   # where the use's remainder stays (see below)
            e = max_rel_err(ds[MONTH_END, i], ex[f"m_{f}_storage"], floor_frac=1e-2)
            errs[f + "_storage"] = 0. if e <= RTOL_WU else e
    days = ex["daily_days"]
    for k in m.DAILY_VERTICAL:
        if k != "land_aet":   # not a grid of the reference's
            errs["d_" + k] = max_rel_err(grids["d_" + k][days], ex["d_" + k])
    if routing:
        for k in m.MONTHLY_ROUTING + ["cell_aet", "cell_aet_wca"]:
            errs[k] = max_rel_err(grids[k], ex["m_" + k])
        if wuse:   # the water use grids are exercised
            assert np.abs(ex["m_actual_use"]).max() > 0 and np.abs(ex["m_nug"]).max() > 0
        for k in m.DAILY_ROUTING:
            if k != "open_water_evap":   # not a grid of the reference's
                errs["d_r_" + k] = max_rel_err(grids["d_r_" + k][days], ex["d_r_" + k])
    if wuse:
        # routing's flux grids with water use: the net abstraction from groundwater
        # can leave a cell's groundwater runoff as a difference of equal terms,
        # zero in the reference and +1e-20 km3 here (or the reverse); the river
        # velocity is not smooth at zero inflow (depth ~ Q^0.341, a floor of 1e-5
        # km/d, routing.cpp:7274-7297), so the day's release differs (cell 149 of
        # this fixture, day 312: 7.5e-8 against 1.3e-9 km3) and the water leaves
        # on the following days instead; every storage and the water-use state
        # agree with the oracle to 1e-14 at the end.  Against a floor of 1 % of each
        # grid's largest value the grids' largest such error is 1.3e-8
        for k in FLUX_WU:
            g = grids[k] if not k.startswith("d_") else grids[k][days]
            r = ex["m_" + ROUTING.get(k, k)] if not k.startswith("d_") else ex[k]
            e = max_rel_err(g, r, floor_frac=1e-2)
            errs[k] = 0. if e <= RTOL_WU else e   # reported (and failing) above RTOL_WU
    bad = {k: v for k, v in errs.items() if not v <= RTOL}
    assert not bad, bad
    q = m.discharge(0, 730)
    if wuse:   # the same transients reach the stations: 2.1e-7 of 1 % of a station's peak
        from test_wuse_oracle import discharge_err
        assert discharge_err(q, ex["discharge"]) <= 1e-6
    else:
        assert max_rel_err(q, ex["discharge"]) <= RTOL


def test_output_grids_deferred_per_day_calls_same_bits():
    """The per-day entry points, queued (wg_set_deferred), give the grids of one
    run bit for bit; without the queue the per-day vertical call is refused
    while the vertical grids are on."""
    _, _, a = _two_years(deferred=False)
    _, _, b = _two_years(deferred=True)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


PATH_WT = os.path.join(os.path.dirname(__file__), "golden", "swb_outputs_wtemp_365d.npz")


@pytest.mark.parametrize("dps,vertical", [(1, True), (5, True), (5, False)])
def test_output_grids_with_water_temperature(dps, vertical):
    """With the water temperature (and so fractional routing): the monthly mean
    temperatures of the river and every water body (-9999 without a computed
    day), routing's aggregates and, in the wavefront's variant with both, the
    vertical balance's grids, against the reference's over one calendar year."""
    from watergap2_gb300.gpu import Model
    from watergap2_gb300.region import load_npz
    region, ex = load_npz(PATH_WT)
    P, T, S = ex["P"], ex["T"], ex["S"]
    nd = P.shape[0]
    m = Model(region, max_days=nd, stations=ex["stations"], days_per_step=dps, water_temp=True)
    m.set_water_temp_inputs(ex["GWT"], region.extras["river_length_file"])
    m.upload_longwave(0, ex["LW"])
    m.monthly_outputs(12, doy_day0=1)
    m.monthly_outputs_vertical(vertical)
    with pytest.raises(Exception):
        m.monthly_outputs_routing(True)                # routing's further grids: not with the water temperature
    m.upload_forcing(0, P, T, S)
    m.run_days(1, 0, nd)
    errs = {}
    for k in m.MONTHLY_WTEMP:
        g, r = m.monthly(k), ex["m_" + k]
        assert np.array_equal(g == -9999., r == -9999.), k   # the same months without a computed temperature
        ok = r != -9999.
        # a temperature is an energy over a heat capacity in K less 273.15: held to
        # 1e-11 of the absolute temperature, as the water-temperature tests hold it
        errs[k] = float(np.max(np.abs(g[ok] - r[ok]) / (np.abs(r[ok]) + 273.15) * (RTOL / 1e-11)))
    errs.update({k: max_rel_err(m.monthly(k), ex["m_" + r]) for k, r in ROUTING.items()})
    if vertical:
        errs.update({k: max_rel_err(m.monthly(k), ex["m_" + k]) for k in m.MONTHLY_VERTICAL})
    bad = {k: v for k, v in errs.items() if not v <= RTOL}
    assert not bad, bad


def test_routing_grids_refused_with_fractional_routing():
    from watergap2_gb300.gpu import Model, WgError
    from watergap2_gb300.region import load_npz
    region, _ = load_npz(PATH)
    m = Model(region.with_options(frac_routing=1), max_days=4)
    with pytest.raises(WgError):
        m.monthly_outputs_routing(True)
    with pytest.raises(WgError):
        m.daily_outputs_routing(4)
    m.monthly_outputs_vertical(True)                   # the vertical balance's grids run with it


def test_daily_grids_refused_without_kc():
    from watergap2_gb300.gpu import Model, WgError
    from watergap2_gb300.region import load_npz
    region, ex = load_npz(PATH)
    region.lct_tables = {k: v for k, v in region.lct_tables.items() if k not in ("kc_min", "kc_max")}
    m = Model(region, max_days=4)
    with pytest.raises(WgError):
        m.daily_outputs_vertical(4)
    m.monthly_outputs(1, doy_day0=1)
    m.monthly_outputs_vertical(True)                   # the monthly grids need no Kc


def test_per_day_vertical_refused_with_vertical_grids():
    from watergap2_gb300.gpu import Model, WgError
    from watergap2_gb300.region import load_npz
    region, ex = load_npz(PATH)
    m = Model(region, max_days=4)
    m.monthly_outputs(1, doy_day0=1)
    m.monthly_outputs_vertical(True)
    m.upload_forcing(0, ex["P"][:4], ex["T"][:4], ex["S"][:4])
    with pytest.raises(WgError):
        m.step_vertical(1, 0)
    m.monthly_outputs_vertical(False)                  # grids off: the per-day call runs
    m.daily_outputs_vertical(4)
    with pytest.raises(WgError):                       # the daily grids refuse it too
        m.step_vertical(1, 0)
    m.daily_outputs_vertical(0)
    m.step_vertical(1, 0)
    m.step_routing(1, 0)


def test_autotune_leaves_the_monthly_sums():
    """The autotuner's trial runs add nothing to the monthly grids: grids after
    tuning equal those of a run without it."""
    from watergap2_gb300.gpu import Model
    from watergap2_gb300.region import load_npz
    region, ex = load_npz(PATH)
    nd = 90
    P, T, S = ex["P"][:nd], ex["T"][:nd], ex["S"][:nd]
    out = []
    for tune in (False, True):
        m = Model(region, max_days=nd, days_per_step=5)
        m.monthly_outputs(3, doy_day0=1)
        m.monthly_outputs_vertical(True)
        m.monthly_outputs_routing(True)
        m.upload_forcing(0, P, T, S)
        if tune:
            assert m.autotune(1, 0, nd, 0, 8)["trials"] > 0
        m.run_days(1, 0, nd)
        out.append({k: m.monthly(k) for k in ["river_avail", "prec", "pet", "open_water_evap", "land_area_frac"]})
    for k in out[0]:
        assert np.allclose(out[0][k], out[1][k], rtol=1e-12, atol=0), k
