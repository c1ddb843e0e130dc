"""The C++ drop-in stand-ins (include/wg_gpu.hpp) in the reference's day loop:
tests/cpp/dropin_loop.cpp runs integrate_wghm_'s loop shape -- calcNewDay for
every cell from an OpenMP loop, routing and updateLandAreaFrac per day, the
month-end reads of the land fraction and the vertical storages -- over two
years, with stand-ins of the reference's state-file classes.  Checked bit for
bit against wg_run_days of the same inputs: the state, every cell's daily
discharge, the state-file cells of the last month (the daily routing storages
the reference writes in routing.cpp:5001-5020 and the month-end vertical
storages of integrateWGHM.cpp:830-847), the additional-output columns and the
snow bands the reference writes on the month's last day."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
YEARS = 2
DFIELDS = ["canopy", "soil", "snow", "lai_precsum", "gw", "river", "loclake", "locwetl", "glolake", "glowetl", "res",
           "rf_loclake", "rf_locwetl", "rf_glolake", "rf_glowetl", "rf_res", "k_release", "laf", "laf_prev",
           "fswb_next"]


def _build(tmp):
    from watergap2_gb300 import gpu
    exe = os.path.join(tmp, "dropin_loop")
    libdir = os.path.dirname(gpu.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-fopenmp", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dropin_loop.cpp"), "-L", libdir, "-lwg_gpu",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    return exe


def _write_case(tmp, region, P, T, S):
    from watergap2_gb300.region import FIELDS
    with open(os.path.join(tmp, "region.bin"), "wb") as f:
        np.array([region.ncell, region.nband, region.river_velo_opt, region.frac_routing], np.int32).tofile(f)
        np.array([region.default_velocity], np.float64).tofile(f)
        for name, _, _ in FIELDS:
            a = np.ascontiguousarray(region.arrays[name])
            np.array([a.nbytes], np.int64).tofile(f)
            a.tofile(f)
    with open(os.path.join(tmp, "forcing.bin"), "wb") as f:
        for x in (P, T, S):
            np.ascontiguousarray(x, np.float32).tofile(f)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_dropin_loop_matches_pipelined_run(tmp_path):
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_small_swb(seed=44)
    n, B = region.ncell, region.nband
    nd = 365 * YEARS
    P, T, S = sy.forcing(region, nd, doy0=1)
    tmp = str(tmp_path)
    _write_case(tmp, region, P, T, S)
    exe = _build(tmp)
    run = subprocess.run([exe, tmp, str(YEARS)], capture_output=True, text=True)
    assert run.returncode == 0, (run.returncode, run.stdout[-2000:], run.stderr[-2000:])
    secs = float(run.stdout.split()[0])
    raw = np.fromfile(os.path.join(tmp, "out.bin"), np.float64)
    o = 0
    got = {}
    for k in DFIELDS:
        got[k] = raw[o:o + n]; o += n
    got["snow_band"] = raw[o:o + n * B]; o += n * B
    q = raw[o:o + nd * n].reshape(nd, n); o += nd * n
    cells = raw[o:o + n * 31 * 10].reshape(n, 31, 10); o += n * 31 * 10
    addout = raw[o:o + n * 53].reshape(n, 53); o += n * 53
    snow_out = raw[o:o + n * 101].reshape(n, 101); o += n * 101
    snow_state = raw[o:o + n * 101].reshape(n, 101); o += n * 101
    assert o == raw.size

    # the same years as one pipelined run per year; December of the last year day
    # by day, its state read after each day
    m = Model(region, max_days=365, stations=np.arange(n))
    qr = np.empty((nd, n))
    daily = []
    for y in range(YEARS):
        sl = slice(365 * y, 365 * (y + 1))
        m.upload_forcing(0, P[sl], T[sl], S[sl])
        if y < YEARS - 1:
            m.run_days(1, 0, 365)
        else:
            m.run_days(1, 0, 334)
            for d in range(334, 365):
                m.step_vertical(d + 1, d)
                m.step_routing(d + 1, d)
                daily.append(m.get_state())
        qr[sl] = m.discharge(0, 365)
    ref = m.get_state()
    assert np.array_equal(q, qr)
    for k in DFIELDS + ["snow_band"]:
        assert np.array_equal(got[k], ref[k]), k
    # December's state-file cells: the day-end routing storages in mm over the
    # continental area, every day (routing.cpp:5001-5020) ...
    area, cf = region.area_km2, region.contfreq
    conv = (area * (cf / 100.)) / 1000000.
    names = ["loclake", "locwetl", "glolake", "glowetl", "res", "river", "gw"]
    for d, st in enumerate(daily):
        for j, k in enumerate(names):
            assert np.array_equal(cells[:, d, 3 + j], st[k] / conv), (d, k)
    # ... and the month-end canopy, snow and soil over the land fraction (integrateWGHM.cpp:840-844)
    laf = ref["laf"]
    for j, k in enumerate(["canopy", "snow", "soil"]):
        assert np.array_equal(cells[:, 0, j], ref[k] * laf / cf), k
    # what calcNewDay writes on the month's last day (daily.cpp:1033-1035, 1258-1262)
    assert np.array_equal(addout[:, 20], ref["soil"]) and np.array_equal(addout[:, 22], ref["canopy"])
    assert np.array_equal(addout[:, 24], ref["snow"])
    bands = ref["snow_band"].reshape(n, B)
    ref_b = bands[:, (np.arange(100) * B) // 100]
    assert np.array_equal(snow_out[:, 1:], ref_b)
    assert np.array_equal(snow_state[:, 1:], np.where(laf[:, None] == 0., 0., ref_b * laf[:, None] / cf[:, None]))
    print(f"drop-in loop: {n} cells x {nd} days in {secs:.3f} s ({n * nd / secs:.3g} cell-days/s)")
