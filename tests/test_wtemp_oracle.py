"""The oracle's water temperature (oracle/wg_wtemp.c) against the reference's own
calcWaterTempClass::calcWTemp (source/calcWaterTemp.cpp), bit for bit, on the
golden records of tests/golden/make_wtemp_golden.py: every water body present
or absent, open water and ice, frozen-through and no-volume cases, cells without
a river, power-plant cooling."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    z = np.load(os.path.join(HERE, "golden", "wtemp_cases.npz"))
    return z["records"], z["out"]


def test_wtemp_restatement_equals_reference_bitwise():
    import oracle
    rec, ref = _golden()
    out = oracle.wtemp(rec)
    same = (out == ref) | (np.isnan(out) & np.isnan(ref))
    assert same.all(), np.argwhere(~same)[:10]


def test_wtemp_golden_records_cover_the_branches():
    rec, ref = _golden()
    t, ice = ref[:, :6], ref[:, 6:]
    assert (t == -9999.).any(axis=0).all()            # every water body absent somewhere
    assert ((t > 0) & (t < 60)).any(axis=0).all()      # and computed somewhere
    assert (t == 0.).any(axis=0).all()                 # frozen or clamped to 0 degC
    assert (ice > 0).any(axis=0).all()                 # ice on every kind of water body
    assert (rec[:, 0] == 1).any()                      # power-plant cooling


def test_oracle_water_temperature_in_routing_matches_reference():
    """The restatement's routing with water temperature against the reference's
    routing.cpp:4241-4513 (harness with calc_wtemp = 1) over a winter with ice,
    run with the reference's 100 snow bands, bit for bit (on the x86-64 host that
    made the fixture): river temperature at the stations every day, and every
    water body's temperature, ice thickness and the river's last outflow at the
    snapshots."""
    from helpers import REF_BANDS, ref_bound, rel_err
    from oracle import Oracle, ref_case
    from watergap2_gb300.region import load_npz
    region, ex = load_npz(os.path.join(HERE, "golden", "swb_wtemp_90d.npz"))
    P, T, S, LW = ex["P"], ex["T"], ex["S"], ex["LW"]
    o = Oracle(region.with_bands(REF_BANDS))
    o.init_water_temp(ex["GWT"])
    bound = ref_bound()
    day, doy = 0, int(ex["doy0"])
    temps = []
    for i, sd in enumerate(int(x) for x in ex["snap_days"]):
        _, dt = o.run_wt(doy, P[day:sd], T[day:sd], S[day:sd], LW[day:sd], daily_temp=True)
        # the state the reference keeps after each day: -9999 becomes the air temperature (>= 0)
        air = np.maximum(T[day:sd].astype(np.float64), 0.0)
        temps.append(np.where(dt == -9999., air, dt))
        doy = (doy - 1 + (sd - day)) % 365 + 1
        day = sd
        for k, f in enumerate(ref_case.WT_FIELDS[:6]):
            assert rel_err(o.wt["temp"][k], ex[f"s{i}_{f}"]) <= bound, f
        for k, f in enumerate(ref_case.WT_FIELDS[6:12]):
            assert rel_err(o.wt["ice"][k], ex[f"s{i}_{f}"]) <= bound, f
        assert rel_err(o.wt["river_avail"], ex[f"s{i}_river_avail"]) <= bound
    got = np.concatenate(temps)[:, ex["stations"]]
    assert rel_err(got, ex["river_temp"]) <= bound
    # the case covers ice on every kind of water body and open rivers
    assert all((ex[f"s1_{f}"] > 0).any() for f in ref_case.WT_FIELDS[6:12])
    assert (ex["river_temp"] > 0).any() and (ex["river_temp"] == 0).any()
