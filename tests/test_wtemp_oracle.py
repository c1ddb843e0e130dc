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
