"""Water use on the GPU (wg_options.water_use: subtract_use = 2, demand met in
the cell itself) against the reference's own code run with the same monthly net
abstractions (tests/golden/swb_wuse_420d.npz; the oracle's restatement is pinned
to it in tests/test_wuse_oracle.py): storages, the water-use state after two
year ends and the stations' discharge, through the wavefront at one and five
days per step, split runs and the per-day entry points; the water balance with
the abstractions closes."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-10   # |GPU - reference| <= TOL * max(|reference|, floor)
STORES = ["gw", "river", "loclake", "locwetl", "glolake", "glowetl", "res", "rf_loclake", "rf_glolake", "rf_res",
          "k_release", "laf", "soil"]


def _case(name="swb_wuse_420d"):
    from watergap2_gb300.region import load_npz
    return load_npz(os.path.join(HERE, "golden", f"{name}.npz"))


def _use(ex):
    return ex["NUS"], ex["NUG"], ex["WDR"], ex["CONS"]


def _model(region, ex, **kw):
    from watergap2_gb300.gpu import Model
    nd, doy0 = ex["P"].shape[0], int(ex["doy0"])
    delayed = "delayed" in ex and bool(ex["delayed"])
    if "GLWD" in ex and "glwd_unit" not in kw:   # aggrNUsGloLakResOpt = 1
        kw["glwd_unit"] = ex["GLWD"]
    m = Model(region, max_days=nd, stations=ex["stations"], water_use=2 if delayed else True, **kw)
    m.set_water_use_inputs(ex["FRGI"])
    m.upload_forcing(0, ex["P"], ex["T"], ex["S"])
    m.upload_water_use_run(0, doy0, nd, _use(ex))
    return m


def _worst(got, ref, floor):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    return float((np.abs(got - ref) / np.maximum(np.abs(ref), floor)).max())


def _check_snapshot(m, ex, i):
    from oracle.ref_case import WU_FIELDS
    st = m.get_state()
    wu = m.water_use()
    bad = {}
    for f in STORES:
        # reduction factors are fractions in [0, 1]: compared absolutely
        e = _worst(st[f], ex[f"s{i}_{f}"], 1.0 if f.startswith("rf_") else 1e-9)
        if not e <= TOL:
            bad[f] = e
    from test_wuse_oracle import WU_FLOOR
    fields = WU_FIELDS + (["wu_unsat_riparian"] if "GLWD" in ex else [])
    for k, f in enumerate(fields):
        e = _worst(wu[k], ex[f"s{i}_{f}"], WU_FLOOR)
        if not e <= TOL:
            bad[f] = e
    assert not bad, (i, bad)


@pytest.mark.parametrize("name", ["swb_wuse_420d", "swb_wuse_frac_200d",    # with fractional routing
                                  "swb_wuse_delayed_420d",                   # delayed satisfaction
                                  # the riparian cells' NUs met by their outflow cell (GLWD units)
                                  "swb_wuse_glwd_420d", "swb_wuse_glwd_delayed_200d"])
@pytest.mark.parametrize("kd", [1, 5])
def test_water_use_matches_reference(name, kd):
    region, ex = _case(name)
    doy0 = int(ex["doy0"])
    m = _model(region, ex, days_per_step=kd)
    prev = 0
    for i, sd in enumerate(ex["snap_days"]):
        sd = int(sd)
        m.run_days((doy0 - 1 + prev) % 365 + 1, prev, sd - prev)
        _check_snapshot(m, ex, i)
        prev = sd
    from test_wuse_oracle import discharge_err
    assert discharge_err(m.discharge(0, prev), ex["discharge"]) <= TOL


def test_water_use_per_day_api_and_split_runs():
    """The per-day entry points and a wavefront run split across calls (chunks of
    seven steps) give the same state as one call."""
    region, ex = _case()
    nd, doy0 = ex["P"].shape[0], int(ex["doy0"])
    a = _model(region, ex, days_per_step=5)
    a.chunk_steps(7)
    total = a.num_steps(nd)
    for lo, hi in ((0, 13), (13, 50), (50, total)):
        a.run_steps(doy0, 0, nd, lo, hi)
    b = _model(region, ex)
    for d in range(nd):
        doy = (doy0 - 1 + d) % 365 + 1
        b.step_vertical(doy, d)
        b.step_routing(doy, d)
    last = len(ex["snap_days"]) - 1
    for m in (a, b):
        _check_snapshot(m, ex, last)


def test_water_use_balance_closes_and_state_round_trips():
    region, ex = _case()
    nd, doy0 = ex["P"].shape[0], int(ex["doy0"])
    m = _model(region, ex, days_per_step=5, record_balance=True)
    s0 = m.balance()[0]
    m.run_days(doy0, 0, nd)
    bal = m.balance()
    total, pin, evap, out, leak, worst = bal
    resid = (total - s0) - (pin - evap - out + leak)
    assert abs(resid) <= 1e-12 * max(abs(total), pin), (resid, total, pin)
    assert worst <= 1e-12, worst
    # net abstractions leave through the evaporation term: more than the run without use
    from watergap2_gb300.gpu import Model
    p = Model(region, max_days=nd, stations=ex["stations"], record_balance=True, days_per_step=5)
    p.upload_forcing(0, ex["P"], ex["T"], ex["S"])
    p.run_days(doy0, 0, nd)
    assert bal[2] > p.balance()[2]
    # checkpoint / restart of the water-use state
    w = m.water_use()
    m.set_water_use(w * 0.5)
    assert np.array_equal(m.water_use(), w * 0.5)


def test_days_without_tables_use_no_water():
    """Forcing days with no uploaded table run without water use: the results equal
    a context without water use."""
    from watergap2_gb300.gpu import Model
    region, ex = _case()
    nd, doy0 = 120, int(ex["doy0"])
    a = Model(region, max_days=nd, stations=ex["stations"], water_use=True, days_per_step=5)
    a.upload_forcing(0, ex["P"][:nd], ex["T"][:nd], ex["S"][:nd])
    a.run_days(doy0, 0, nd)
    b = Model(region, max_days=nd, stations=ex["stations"], days_per_step=5)
    b.upload_forcing(0, ex["P"][:nd], ex["T"][:nd], ex["S"][:nd])
    b.run_days(doy0, 0, nd)
    sa, sb = a.get_state(), b.get_state()
    for f in STORES:
        assert np.array_equal(sa[f], sb[f]), f
    assert np.array_equal(a.discharge(0, nd), b.discharge(0, nd))


def test_water_use_with_temperature_matches_reference():
    """Water use together with the water temperature (k_pipeline<double,...,3>)
    against the reference run with both (tests/golden/swb_wtemp_wuse_120d.npz)."""
    from oracle.ref_case import WT_FIELDS, WU_FIELDS
    from test_wuse_oracle import discharge_err
    from watergap2_gb300.gpu import Model
    region, ex = _case("swb_wtemp_wuse_120d")
    nd, doy0 = ex["P"].shape[0], int(ex["doy0"])
    m = Model(region, max_days=nd, stations=ex["stations"], water_use=True, water_temp=True, days_per_step=5)
    m.set_water_use_inputs(ex["FRGI"])
    m.set_water_temp_inputs(ex["GWT"], region.extras["river_length_file"])
    m.upload_forcing(0, ex["P"], ex["T"], ex["S"])
    m.upload_longwave(0, ex["LW"])
    m.upload_water_use_run(0, doy0, nd, _use(ex))
    prev = 0
    for i, sd in enumerate(ex["snap_days"]):
        sd = int(sd)
        m.run_days((doy0 - 1 + prev) % 365 + 1, prev, sd - prev)
        temp, ice = m.water_temp()
        wu = m.water_use()
        st = m.get_state()
        bad = {}
        for k in range(6):
            if not _worst(temp[k], ex[f"s{i}_{WT_FIELDS[k]}"], 1.0) <= TOL:
                bad[WT_FIELDS[k]] = _worst(temp[k], ex[f"s{i}_{WT_FIELDS[k]}"], 1.0)
            if not _worst(ice[k], ex[f"s{i}_{WT_FIELDS[6 + k]}"], 1e-9) <= TOL:
                bad[WT_FIELDS[6 + k]] = _worst(ice[k], ex[f"s{i}_{WT_FIELDS[6 + k]}"], 1e-9)
        for k, f in enumerate(WU_FIELDS):
            if not _worst(wu[k], ex[f"s{i}_{f}"], 1e-9) <= TOL:
                bad[f] = _worst(wu[k], ex[f"s{i}_{f}"], 1e-9)
        for f in ("river", "soil", "gw", "loclake", "glolake", "res"):
            if not _worst(st[f], ex[f"s{i}_{f}"], 1e-9) <= TOL:
                bad[f] = _worst(st[f], ex[f"s{i}_{f}"], 1e-9)
        assert not bad, (i, bad)
        prev = sd
    assert discharge_err(m.discharge(0, nd), ex["discharge"]) <= TOL
    assert _worst(m.river_temp(0, nd), ex["river_temp"], 1.0) <= TOL


def test_water_use_fp32_and_ensemble():
    """Water use in FP32 state (FP64 sums) stays close to the FP64 run, and an
    ensemble of identical members gives each member the single FP32 run's bits."""
    region, ex = _case()
    nd, doy0 = ex["P"].shape[0], int(ex["doy0"])
    ref = _model(region, ex, days_per_step=5)
    ref.run_days(doy0, 0, nd)
    f32 = _model(region, ex, days_per_step=5, precision="fp32")
    f32.run_days(doy0, 0, nd)
    q64, q32 = ref.discharge(0, nd), f32.discharge(0, nd)
    # where demand takes nearly a river's whole flow, the remainder is a small
    # difference that FP32 rounding moves (as the fine-resolution run's threshold
    # branches do): the run's volumes and the typical day stay close
    peak = np.abs(q64).max(axis=0, keepdims=True)
    daily = np.abs(q32 - q64) / np.maximum(np.abs(q64), 1e-2 * peak + 1e-12)
    vol = np.abs(q32.sum(axis=0) - q64.sum(axis=0)) / np.maximum(q64.sum(axis=0), 1e-12)
    w64, w32 = ref.water_use(), f32.water_use()
    use = abs(w32[11].sum() - w64[11].sum()) / abs(w64[11].sum())
    stats = dict(daily_median=float(np.median(daily)), daily_q99=float(np.quantile(daily, 0.99)),
                 volume_max=float(vol.max()), actual_use=float(use))
    # measured on GB300: median 4.6e-7, volume 1.3 % at the station whose river the
    # fixture's demand nearly empties, actual use 5e-4
    assert stats["daily_median"] < 1e-5 and stats["volume_max"] < 0.05 and stats["actual_use"] < 1e-3, stats
    M = 4
    ens = _model(region, ex, days_per_step=5, precision="fp32", members=M)
    ens.run_days(doy0, 0, nd)
    qe = ens.discharge(0, nd)                        # [days, stations, members]
    we = ens.water_use()                             # [12, ncell, members]
    for mm in range(M):
        assert np.array_equal(qe[:, :, mm], q32)
        assert np.array_equal(we[:, :, mm], w32)


def test_glwd_per_day_api_and_split_runs():
    """With GLWD units: the per-day entry points and a wavefront run split across
    calls reach the reference's state of the last snapshot."""
    region, ex = _case("swb_wuse_glwd_420d")
    nd, doy0 = ex["P"].shape[0], int(ex["doy0"])
    a = _model(region, ex, days_per_step=5)
    a.chunk_steps(7)
    total = a.num_steps(nd)
    for lo, hi in ((0, 13), (13, 50), (50, total)):
        a.run_steps(doy0, 0, nd, lo, hi)
    b = _model(region, ex)
    for d in range(nd):
        doy = (doy0 - 1 + d) % 365 + 1
        b.step_vertical(doy, d)
        b.step_routing(doy, d)
    last = len(ex["snap_days"]) - 1
    for m in (a, b):
        _check_snapshot(m, ex, last)


def _global_errors(region, P, T, S, use, frgi, unit, nd):
    """Per-cell relative errors of the GPU (the bench's launch set-up) against the
    oracle: storages, water-use rows and the outlets' discharge."""
    import os as _os
    from oracle import Oracle
    from test_wuse_oracle import WU_FLOOR
    from watergap2_gb300.gpu import Model
    outlets = np.nonzero(region.downstream < 0)[0]
    m = Model(region, max_days=nd, stations=outlets, water_use=True, glwd_unit=unit, days_per_step=5)
    assert m.vertical_overlap() > 0 and m.chunk_steps() == 4
    m.set_water_use_inputs(frgi)
    m.upload_forcing(0, P, T, S)
    m.upload_water_use_run(0, 1, nd, use)
    m.run_days(1, 0, nd)
    st, wu, q = m.get_state(), m.water_use(), m.discharge(0, nd)
    del m
    o = Oracle(region)
    o.init_water_use(frgi, glwd_unit=unit)
    qo, _, _ = o.run_wu(1, P, T, S, use, discharge=True, nthreads=_os.cpu_count() or 1)
    rel = lambda a, b, fl: np.abs(np.asarray(a) - b) / np.maximum(np.abs(b), fl)
    err = {f: rel(st[f], o.state[f], 1.0 if f.startswith("rf_") else 1e-9) for f in STORES}
    for k in range(wu.shape[0]):
        err[f"wu{k}"] = rel(wu[k], o.wu[k], WU_FLOOR)
    qr = qo[:, outlets]
    err["discharge"] = (np.abs(q - qr) / np.maximum(np.abs(qr), np.maximum(1e-2 * np.abs(qr).max(axis=0), 1e-9))).max(axis=0)
    return err, o.wu


def test_glwd_global_grid_as_benchmarked_vs_oracle():
    """The global grid with water use and the riparian cells of its 1,500 global
    lakes and reservoirs (5,781 cells in GLWD units) met by their outflow cells,
    in the bench's launch set-up (five days per step, four-step chunks, the
    vertical-balance warps), over a year with heavy riparian demand, against the
    oracle: every storage and the riparian cells' share of unmet use within
    1e-10.  The water-use state and the discharge hold 1e-10 too, except at the
    few cells where the run without units differs from the oracle by as much:
    a headwater cell whose river the abstraction empties routes a residue of
    runoff minus recharge, and the velocity of variable-velocity routing grows
    with that inflow to the power 0.227 (getRiverVelocity, routing.cpp:7274-7306),
    so ulp differences of exp and pow move the day's split between storage and
    outflow.  The units add no difference of their own."""
    from watergap2_gb300 import synthetic as sy
    region = sy.region_global()
    unit = sy.glwd_units(region)
    nd = 365
    P, T, S = sy.forcing(region, nd, seed=2, doy0=1)
    nus, nug, wdr, cons, frgi = sy.water_use_inputs(region, 2, seed=5)
    rip = np.nonzero((unit > 0) & (region.lake_area <= 0) & (region.res_area <= 0))[0]
    nus = nus.copy()
    nus[:, :, rip] = (np.abs(nus[:, :, rip]) * 30.0 + np.float32(5.0e8)).astype(np.float32)
    use = (nus, nug, wdr, cons)
    eg, owu = _global_errors(region, P, T, S, use, frgi, unit, nd)
    ep, _ = _global_errors(region, P, T, S, use, frgi, None, nd)
    print("GLWD global year: riparian shares > 0:", int((owu[12] > 0).sum()),
          {k: f"{v.max():.2e}/{ep[k].max():.2e}" for k, v in eg.items() if k in ep and v.max() > 1e-12})
    assert (owu[12] > 0).sum() > 100
    bad = {}
    for k, e in eg.items():
        if k in STORES or k == "wu12":
            ok = e <= TOL
        else:   # beyond 1e-10 only where the run without units differs as much
            ok = (e <= TOL) | (e <= 1.01 * ep[k])
        if not ok.all():
            bad[k] = (float(e.max()), int((~ok).sum()))
    assert not bad, bad
    assert max(ep[k].max() for k in STORES) <= TOL
