"""The CPU oracle against the reference's own outputs (golden fixtures).

The fixtures in tests/golden/ hold inputs and the results of the reference's
calcNewDay/routing object code (made by tests/golden/make_golden.py).  The C
restatement reproduces them bit for bit on the x86 host that made them; on
other hosts libm may round differently in the last place, hence the 1e-12
relative bound.  The fixtures were made with the reference's 100 bands (each of
the 5 synthetic bands replicated 20 times); the restatement runs the 5 bands, so
band sums differ from the reference's only in rounding.
"""
import glob
import os

import numpy as np
import pytest

from oracle import Oracle
from watergap2_gb300.region import load_npz

FIXTURES = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                  if not ({"wtemp", "wuse"} & set(os.path.basename(p)[:-4].split("_"))))   # test_wtemp_oracle.py, test_wuse_oracle.py
STATE_KEYS = ["canopy", "soil", "snow", "lai_days", "lai_status", "lai_precsum", "gw", "river", "loclake",
              "locwetl", "glolake", "glowetl", "res", "rf_loclake", "rf_locwetl", "rf_glolake", "rf_glowetl",
              "rf_res", "k_release", "laf", "laf_prev"]


def rel_err(a, b, floor=1e-30):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.maximum(np.abs(b), floor)
    return float(np.max(np.abs(a - b) / scale)) if a.size else 0.0


def test_fixtures_present():
    assert len(FIXTURES) >= 4


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_reference(path):
    region, ex = load_npz(path)
    P, T, S = ex["P"], ex["T"], ex["S"]
    doy0 = int(ex["doy0"])
    snaps = [int(x) for x in ex["snap_days"]]
    o = Oracle(region)
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
            # tiny storages are compared absolutely (km3 / mm near the 1e-15 snapping limit)
            err = np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-9)) if ref.size else 0.0
            assert err <= 1e-12, (k, err)
        got_b = o.state["snow_band"].reshape(region.ncell, region.nband)
        assert np.max(np.abs(got_b - ex[f"s{i}_snow_band"]) / np.maximum(np.abs(ex[f"s{i}_snow_band"]), 1e-9)) <= 1e-12
    q = np.concatenate(q_all)[:, ex["stations"]]
    ref_q = ex["discharge"][: q.shape[0]]
    assert np.max(np.abs(q - ref_q) / np.maximum(np.abs(ref_q), 1e-12)) <= 1e-12


@pytest.mark.parametrize("path", FIXTURES[:2], ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_mass_balance_closes(path):
    region, ex = load_npz(path)
    o = Oracle(region)
    _, b = o.run(int(ex["doy0"]), ex["P"], ex["T"], ex["S"], balance=True)
    resid = np.abs(b[:, 5])
    assert np.max(resid / b[:, 0]) < 1e-12
