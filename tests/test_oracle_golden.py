"""The CPU oracle against the reference's own outputs (golden fixtures).

The fixtures in tests/golden/ hold inputs and the results of the reference's
calcNewDay/routing object code (made by tests/golden/make_golden.py); the
workloads too large to store keep their seeds, a digest of the regenerated
inputs and the reference's outputs.  The reference runs 100 snow bands (each of
the 5 synthetic bands replicated 20 times); the oracle, run with the same 100
bands, reproduces every output bit for bit on the x86-64 host that made the
fixtures (elsewhere libm may round a transcendental differently in the last
place: 1e-12 relative).
"""
import glob
import os

import numpy as np
import pytest

from oracle import Oracle
from watergap2_gb300.region import load_npz

FIXTURES = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                  if not ({"wtemp", "wuse", "glwd"} & set(os.path.basename(p)[:-4].split("_")))
                  and not os.path.basename(p).startswith("config"))   # regenerated workloads: own tests   # test_wtemp_oracle.py, test_wuse_oracle.py
STATE_KEYS = ["canopy", "soil", "snow", "lai_days", "lai_status", "lai_precsum", "gw", "river", "loclake",
              "locwetl", "glolake", "glowetl", "res", "rf_loclake", "rf_locwetl", "rf_glolake", "rf_glowetl",
              "rf_res", "k_release", "laf", "laf_prev"]


def test_fixtures_present():
    assert len(FIXTURES) >= 4


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_reference(path):
    from helpers import REF_BANDS, ref_bound, rel_err
    region, ex = load_npz(path)
    P, T, S = ex["P"], ex["T"], ex["S"]
    doy0 = int(ex["doy0"])
    snaps = [int(x) for x in ex["snap_days"]]
    rep = REF_BANDS // region.nband
    o = Oracle(region.with_bands(REF_BANDS))
    bound = ref_bound()
    q_all = []
    day = 0
    doy = doy0
    for i, sd in enumerate(snaps):
        q, _ = o.run(doy, P[day:sd], T[day:sd], S[day:sd], discharge=True)
        q_all.append(q)
        doy = (doy - 1 + (sd - day)) % 365 + 1
        day = sd
        for k in STATE_KEYS:
            ref = ex[f"s{i}_{k}"]
            got = o.state[k]
            if k == "k_release":   # only defined in reservoir cells (routing.cpp:443-446)
                m = region.res_area > 0
                ref, got = ref[m], got[m]
            assert rel_err(got, ref) <= bound, k
        got_b = o.state["snow_band"].reshape(region.ncell, region.nband, rep)[:, :, 0]
        assert rel_err(got_b, ex[f"s{i}_snow_band"]) <= bound
    q = np.concatenate(q_all)[:, ex["stations"]]
    assert rel_err(q, ex["discharge"][: q.shape[0]]) <= bound


@pytest.mark.parametrize("path", FIXTURES[:2], ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_mass_balance_closes(path):
    region, ex = load_npz(path)
    o = Oracle(region)
    _, b = o.run(int(ex["doy0"]), ex["P"], ex["T"], ex["S"], balance=True)
    resid = np.abs(b[:, 5])
    assert np.max(resid / b[:, 0]) < 1e-12


def test_oracle_balance_closes_without_continental_area():
    """Cells without continental area (swb_nocont_150d) route nothing: the inflow
    they receive leaves the system as a negative leak, and the balance still
    closes every day."""
    region, ex = load_npz(os.path.join(os.path.dirname(__file__), "golden", "swb_nocont_150d.npz"))
    o = Oracle(region)
    _, b = o.run(int(ex["doy0"]), ex["P"], ex["T"], ex["S"], balance=True)
    assert np.max(np.abs(b[:, 5]) / b[:, 0]) < 1e-12
    assert np.sum(b[:, 4]) < 0.   # inflow into the cells without continental area


def _regen_module():
    import importlib.util
    path = os.path.join(os.path.dirname(__file__), "golden", "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


REGEN = ["config1_region64_365d", "config2_global_120d"]


@pytest.mark.parametrize("name", REGEN)
def test_oracle_matches_reference_on_workload(name):
    """The 64 x 64 region over a year and the 67,420-cell global grid with every
    kind of water body over 120 days, inputs regenerated from their seeds: the
    oracle, run with the reference's 100 snow bands (each of the 5 synthetic
    bands 20 times), against the reference's stations, sampled cells and exact
    sums over all cells -- bit for bit."""
    from helpers import REF_BANDS, field_sums, input_digest, ref_bound, rel_err
    mg = _regen_module()
    ex = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))
    region, P, T, S, doy0, snaps, sample, stations = mg.regen_inputs(name)
    if input_digest(region, P, T, S) != str(ex["digest"]):
        pytest.fail(f"{name}: the seeded generators drew different inputs on this host (numpy {np.__version__})")
    assert np.array_equal(stations, ex["stations"]) and np.array_equal(sample, ex["sample"])
    keys = [str(k) for k in ex["keys"]]
    rep = REF_BANDS // region.nband
    o = Oracle(region.with_bands(REF_BANDS))
    bound = ref_bound()
    q_all, day, doy = [], 0, doy0
    for i, sd in enumerate(snaps):
        q, _ = o.run(doy, P[day:sd], T[day:sd], S[day:sd], discharge=True, nthreads=os.cpu_count() or 1)
        q_all.append(q[:, stations])
        doy = (doy - 1 + (sd - day)) % 365 + 1
        day = sd
        bands = o.state["snow_band"].reshape(region.ncell, region.nband, rep)
        st = dict(o.state, snow_band=bands[:, :, 0])
        assert rel_err(field_sums(st, keys + ["snow_band"]), ex[f"s{i}_sums"]) <= bound, i
        if f"s{i}_soil" in ex:
            for k in keys + ["snow_band", "k_release"]:
                ref, got = ex[f"s{i}_{k}"], st[k][sample]
                if k == "k_release":   # only defined in reservoir cells (routing.cpp:443-446)
                    m = region.res_area[sample] > 0
                    ref, got = ref[m], got[m]
                assert rel_err(got, ref) <= bound, k
    assert rel_err(np.concatenate(q_all), ex["discharge"]) <= bound


def test_station_correction_fixture_changes_discharge():
    """The statcorrOpt fixture exercises the correction: without it the oracle's
    station discharge differs from the reference's."""
    region, ex = load_npz(os.path.join(os.path.dirname(__file__), "golden", "swb_statcorr_120d.npz"))
    assert region.statcorr_opt == 1 and np.any(region.param("P_CFS") != 1.0)
    o = Oracle(region.with_options(statcorr_opt=0).with_bands(100))
    q, _ = o.run(int(ex["doy0"]), ex["P"], ex["T"], ex["S"], discharge=True)
    assert not np.allclose(q[:, ex["stations"]], ex["discharge"], rtol=1e-6)


def test_output_fixture_pinned_to_its_inputs():
    """The reference's grids in swb_outputs_730d are its second year's month sums
    and day values in cell order (grid_store = 6 divides the means only when it
    writes): monthly precipitation and temperature equal the sums of the
    fixture's daily forcing exactly, the daily ones the forcing itself, and the
    month-end storages at December's end equal the state of the same run's
    day-730 snapshot."""
    region, ex = load_npz(os.path.join(os.path.dirname(__file__), "golden", "swb_outputs_730d.npz"))
    b = 365 + np.r_[0, np.cumsum([31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31])]
    days = ex["daily_days"]
    for f, field in (("prec", "P"), ("temp", "T")):
        x = ex[field].astype(np.float64)
        sums = np.array([x[b[k]:b[k + 1]].sum(axis=0) for k in range(12)])
        assert np.array_equal(sums, ex[f"m_{f}"]), f
        assert np.array_equal(x[365 + days], ex[f"d_{f}"]), f
    for f in ("loclake", "locwetl", "glolake", "glowetl", "res", "river", "gw"):
        assert np.array_equal(ex[f"m_{f}_storage"][11], ex[f"s0_{f}"]), f
