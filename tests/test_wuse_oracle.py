"""The oracle's water use (subtract_use = 2, demand satisfied in the cell itself)
against the reference's own daily.cpp/routing.cpp run with the same monthly net
abstractions (tests/golden/swb_wuse_420d.npz, made by tests/golden/make_golden.py):
every storage, the water-use state of routingClass (remaining and unsatisfied
use, reduced return flows, the previous year's values after two year ends) and
the stations' discharge."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "swb_wuse_420d.npz")
FIXTURES = [FIXTURE, os.path.join(HERE, "golden", "swb_wuse_frac_200d.npz"),   # with fractional routing
            os.path.join(HERE, "golden", "swb_wuse_delayed_420d.npz"),         # delayed satisfaction
            # the NUs of global lakes' and reservoirs' riparian cells met by their outflow cell
            # (aggrNUsGloLakResOpt = 1), without and with delayed satisfaction
            os.path.join(HERE, "golden", "swb_wuse_glwd_420d.npz"),
            os.path.join(HERE, "golden", "swb_wuse_glwd_delayed_200d.npz")]
STORES = ["gw", "river", "loclake", "locwetl", "glolake", "glowetl", "res", "rf_loclake", "rf_glolake", "rf_res",
          "k_release", "laf", "soil"]


def _load(path=FIXTURE):
    from watergap2_gb300.region import load_npz
    return load_npz(path)


def _close(got, ref, floor, tol=1e-10):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    err = np.abs(got - ref) / np.maximum(np.abs(ref), floor)
    return float(err.max()) if err.size else 0.0


def discharge_err(q, ref):
    """Largest |q - ref| / max(|ref|, 1 % of the station's peak): where the river
    meets a use close to its whole flow, the small remainder carries the
    cancellation of that subtraction (rounding of the reference's 100 snow bands
    against the restatement's 5 at the 1e-15 km3 level)."""
    ref = np.asarray(ref, np.float64)
    floor = np.maximum(1e-2 * np.abs(ref).max(axis=0, keepdims=True), 1e-9)
    return float((np.abs(np.asarray(q) - ref) / np.maximum(np.abs(ref), floor)).max())


# water-use volumes [km3] are compared against max(|value|, 1e-6 km3 = 1,000 m3):
# the remaining use is a difference of nearly equal volumes every day (delayed
# satisfaction subtracts the previous day's unmet demand), so values of 1e-18 km3
# differ in their leading digits
WU_FLOOR = 1e-6


def _use(ex):
    return ex["NUS"], ex["NUG"], ex["WDR"], ex["CONS"]


def test_fixture_exercises_water_use():
    region, ex = _load()
    from oracle.ref_case import WU_FIELDS
    last = len(ex["snap_days"]) - 1
    # unmet demand, adapted groundwater abstraction and both year-end branches occur
    assert any(np.any(ex[f"s{i}_wu_remaining"] > 0) for i in range(last + 1))
    assert np.any(ex[f"s{last}_wu_reduced_return"] != 0)
    assert np.any(ex[f"s{last}_wu_unsat_prev"] > 0)
    assert np.any(ex["NUS"] < 0) and np.any(ex["NUG"] < 0)
    assert (ex[f"s{last}_loclake"] < 0).any()          # local lakes drawn below zero by abstraction
    assert (ex[f"s{last}_glolake"] < 0).any()          # and global lakes
    for f in WU_FIELDS:
        assert f"s0_{f}" in ex


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
@pytest.mark.parametrize("nthreads", [1, 4])
def test_oracle_water_use_matches_reference(path, nthreads):
    """Bit for bit (on the x86-64 host that made the fixtures), the oracle run
    with the reference's 100 snow bands: storages, the water-use state values
    (with GLWD units also G_unsatUseRiparian) at every snapshot and the stations'
    daily discharge."""
    import oracle
    from helpers import REF_BANDS, ref_bound, rel_err
    from oracle.ref_case import WU_FIELDS
    region, ex = _load(path)
    doy0 = int(ex["doy0"])
    P, T, S = ex["P"], ex["T"], ex["S"]
    worst = {}
    prev = 0
    o = oracle.Oracle(region.with_bands(REF_BANDS))
    glwd = ex["GLWD"] if "GLWD" in ex else None
    o.init_water_use(ex["FRGI"], delayed=bool(ex["delayed"]) if "delayed" in ex else False, glwd_unit=glwd)
    fields = WU_FIELDS + (["wu_unsat_riparian"] if glwd is not None else [])
    qs = []
    for i, sd in enumerate(ex["snap_days"]):
        sd = int(sd)
        # continue the same run: the call's year index restarts, so pass the tables from its own year on
        d0doy = (doy0 - 1 + prev) % 365 + 1
        years_done = int(np.sum(((doy0 - 1 + np.arange(1, prev + 1)) % 365 + 1) == 1)) if prev else 0
        use = tuple(u[years_done:] for u in _use(ex))
        q, b, _ = o.run_wu(d0doy, P[prev:sd], T[prev:sd], S[prev:sd], use, discharge=True, balance=True,
                           nthreads=nthreads)
        qs.append(q)
        assert np.abs(b[:, 5]).max() < 1e-9 * max(1.0, np.abs(b[:, 0]).max())
        for f in STORES:
            worst[f] = max(worst.get(f, 0.0), rel_err(o.state[f], ex[f"s{i}_{f}"]))
        for k, f in enumerate(fields):
            worst[f] = max(worst.get(f, 0.0), rel_err(o.wu[k], ex[f"s{i}_{f}"]))
        prev = sd
    q = np.concatenate(qs)[:, ex["stations"]]
    worst["discharge"] = rel_err(q, ex["discharge"])
    bad = {k: v for k, v in worst.items() if not v <= ref_bound()}
    assert not bad, bad


def test_oracle_water_use_with_temperature_matches_reference():
    """Water use and the water temperature together (tests/golden/swb_wtemp_wuse_120d.npz:
    a cold season across a year end, ice on the water bodies, lakes drawn down);
    bit for bit as above."""
    import oracle
    from helpers import REF_BANDS, ref_bound, rel_err
    from oracle.ref_case import WT_FIELDS, WU_FIELDS
    from watergap2_gb300.region import load_npz
    region, ex = load_npz(os.path.join(HERE, "golden", "swb_wtemp_wuse_120d.npz"))
    o = oracle.Oracle(region.with_bands(REF_BANDS))
    o.init_water_temp(ex["GWT"])
    o.init_water_use(ex["FRGI"])
    doy0, prev = int(ex["doy0"]), 0
    worst = {}
    for i, sd in enumerate(ex["snap_days"]):
        sd = int(sd)
        years_done = int(np.sum(((doy0 - 1 + np.arange(1, prev + 1)) % 365 + 1) == 1)) if prev else 0
        use = tuple(u[years_done:] for u in _use(ex))
        o.run_wt_wu((doy0 - 1 + prev) % 365 + 1, ex["P"][prev:sd], ex["T"][prev:sd], ex["S"][prev:sd],
                    ex["LW"][prev:sd], use)
        for k in range(6):
            for arr, f in ((o.wt["temp"][k], WT_FIELDS[k]), (o.wt["ice"][k], WT_FIELDS[6 + k])):
                worst[f] = max(worst.get(f, 0.0), rel_err(arr, ex[f"s{i}_{f}"]))
        for k, f in enumerate(WU_FIELDS):
            worst[f] = max(worst.get(f, 0.0), rel_err(o.wu[k], ex[f"s{i}_{f}"]))
        for f in ("river", "soil", "gw", "loclake", "glolake", "res"):
            worst[f] = max(worst.get(f, 0.0), rel_err(o.state[f], ex[f"s{i}_{f}"]))
        prev = sd
    bad = {k: v for k, v in worst.items() if not v <= ref_bound()}
    assert not bad, bad
    assert (ex["s1_ice_river"] > 0).any() and (ex["s1_wu_actual"] != 0).any()


def test_glwd_fixtures_exercise_the_aggregation():
    """The GLWD fixtures reach every branch that matters: aggregated use left
    unmet and handed back to riparian cells (G_unsatUseRiparian > 0) at the
    snapshots, riparian cells upstream and downstream of their outflow cell,
    and riparian cells that return water (negative NUs)."""
    for name in ("swb_wuse_glwd_420d", "swb_wuse_glwd_delayed_200d"):
        region, ex = _load(os.path.join(HERE, "golden", f"{name}.npz"))
        unit = ex["GLWD"]
        outflow = (region.lake_area > 0) | (region.res_area > 0)
        assert np.all(unit[outflow] > 0)
        rip = (unit > 0) & ~outflow
        down = region.downstream
        assert any(down[i] >= 0 and outflow[down[i]] for i in np.nonzero(rip)[0])         # upstream riparian
        assert any(down[c] >= 0 and rip[down[c]] for c in np.nonzero(outflow)[0])        # downstream riparian
        assert (ex["NUS"][..., rip] < 0).any()
        assert any((ex[f"s{i}_wu_unsat_riparian"] > 0).any() for i in range(len(ex["snap_days"])))


def test_aggregate_nus_refuses_what_the_reference_would_mangle():
    """An outflow cell without a unit would aggregate every cell without one, and
    two outflow cells in one unit would aggregate it twice: both are refused."""
    from oracle import aggregate_nus
    from watergap2_gb300 import synthetic as sy
    region, ex = _load(os.path.join(HERE, "golden", "swb_wuse_glwd_420d.npz"))
    unit = ex["GLWD"].copy()
    nus = ex["NUS"][:1].astype(np.float64)
    agg = aggregate_nus(region, unit, nus)
    outflow = np.nonzero((region.lake_area > 0) | (region.res_area > 0))[0]
    # the unit's positive NUs end in the outflow cell; the totals stay
    assert np.allclose(agg.sum(axis=-1), nus.sum(axis=-1), rtol=1e-12)
    moved = (unit > 0) & (nus[0, 0] > 0) & ~np.isin(np.arange(region.ncell), outflow)
    assert np.all(agg[0, 0, moved] == 0)
    bad = unit.copy()
    bad[outflow[0]] = 0
    with pytest.raises(ValueError):
        aggregate_nus(region, bad, nus)
    bad = unit.copy()
    bad[outflow[1]] = bad[outflow[0]]
    with pytest.raises(ValueError):
        aggregate_nus(region, bad, nus)
    assert sy.glwd_units(region).tolist() == unit.tolist()
