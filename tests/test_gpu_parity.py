"""GPU (libwg_gpu.so through its C ABI) against the reference and the oracle.

* golden fixtures: outputs of the reference's own code (tests/golden/);
* the CPU oracle on the same seeded inputs, generated here: the 64 x 64 FP64
  region over a full year, a region with every water-body type over two years,
  and the 67,420-cell global grid over two months;
* internal consistency: the day-pipelined launch equals the per-day entry
  points bit for bit, chunked runs equal one run, and a state saved and
  restored continues identically.

Tolerance (FP64 path): 1e-10 relative on every storage and on discharge.
"""
import glob
import os

import numpy as np
import pytest

from helpers import STATE_KEYS, STORAGES, max_rel_err, state_errors

pytestmark = pytest.mark.gpu
RTOL = 1e-10
FIXTURES = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                  if not ({"wtemp", "wuse", "glwd"} & set(os.path.basename(p)[:-4].split("_")))
                  and not os.path.basename(p).startswith("config"))   # regenerated workloads: own tests   # test_gpu_wtemp.py, test_gpu_wuse.py


@pytest.fixture(scope="module", autouse=True)
def _built():
    from watergap2_gb300 import build, gpu
    if not os.path.exists(gpu.LIB_PATH):
        build.build()


def _model(region, **kw):
    from watergap2_gb300.gpu import Model
    return Model(region, **kw)


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_matches_reference_fixture(path):
    from watergap2_gb300.region import load_npz
    region, ex = load_npz(path)
    P, T, S = ex["P"], ex["T"], ex["S"]
    doy0 = int(ex["doy0"])
    m = _model(region, max_days=P.shape[0], stations=ex["stations"])
    m.upload_forcing(0, P, T, S)
    day, doy = 0, doy0
    for i, sd in enumerate(int(x) for x in ex["snap_days"]):
        m.run_days(doy, day, sd - day)
        doy = (doy - 1 + (sd - day)) % 365 + 1
        day = sd
        got = m.get_state()
        ref = {k: ex[f"s{i}_{k}"] for k in STATE_KEYS if f"s{i}_{k}" in ex}
        errs = state_errors(got, ref, keys=[k for k in ref if k != "k_release"])
        assert max(errs.values()) <= RTOL, errs
        gb = got["snow_band"].reshape(region.ncell, region.nband)
        assert max_rel_err(gb, ex[f"s{i}_snow_band"]) <= RTOL
    q = m.discharge(0, P.shape[0])
    assert max_rel_err(q, ex["discharge"]) <= RTOL


def _oracle_vs_gpu(region, nd, doy0, seed=2, per_day=False):
    from oracle import Oracle
    from watergap2_gb300 import synthetic as sy
    P, T, S = sy.forcing(region, nd, seed=seed, doy0=doy0)
    o = Oracle(region)
    qo, _ = o.run(doy0, P, T, S, discharge=True)
    m = _model(region, max_days=min(nd, 400), stations=np.arange(region.ncell))
    qg = m.run(doy0, P, T, S, per_day=per_day)
    got = m.get_state()
    errs = state_errors(got, o.state)
    errs["discharge"] = max_rel_err(qg, qo)
    errs["snow_band"] = max_rel_err(got["snow_band"], o.state["snow_band"])
    return errs


def test_region64_full_year_vs_oracle():
    from watergap2_gb300 import synthetic as sy
    errs = _oracle_vs_gpu(sy.region_64x64(), 365, 1)
    assert max(errs.values()) <= RTOL, errs


def test_water_bodies_two_years_vs_oracle():
    from watergap2_gb300 import synthetic as sy
    errs = _oracle_vs_gpu(sy.region_small_swb(seed=31), 730, 45)
    assert max(errs.values()) <= RTOL, errs


def test_storage_based_velocity_vs_oracle():
    from watergap2_gb300 import synthetic as sy
    errs = _oracle_vs_gpu(sy.region_small_swb(seed=8, river_velo_opt=2), 200, 100)
    assert max(errs.values()) <= RTOL, errs


def test_global_grid_two_months_vs_oracle():
    from watergap2_gb300 import synthetic as sy
    errs = _oracle_vs_gpu(sy.region_global(), 60, 150)
    assert max(errs.values()) <= RTOL, errs


def test_pipelined_launch_equals_per_day_calls():
    from watergap2_gb300 import synthetic as sy
    region = sy.region_small_swb(seed=12)
    P, T, S = sy.forcing(region, 90, doy0=200)
    a = _model(region, max_days=90)
    qa = a.run(200, P, T, S, per_day=True)
    b = _model(region, max_days=90)
    qb = b.run(200, P, T, S)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    assert np.array_equal(qa, qb)


def test_chunked_run_equals_single_run():
    from watergap2_gb300 import synthetic as sy
    region = sy.region_64x64(seed=4, size=32)
    P, T, S = sy.forcing(region, 120, doy0=300)
    a = _model(region, max_days=120)
    qa = a.run(300, P, T, S)
    b = _model(region, max_days=30)
    qb = b.run(300, P, T, S, chunk=30)
    assert np.array_equal(qa, qb)
    for k, v in a.get_state().items():
        assert np.array_equal(v, b.get_state()[k]), k


def test_state_save_restore_resumes_identically():
    from watergap2_gb300 import synthetic as sy
    region = sy.region_small_swb(seed=13)
    P, T, S = sy.forcing(region, 80, doy0=10)
    a = _model(region, max_days=80)
    qa = a.run(10, P, T, S)
    b = _model(region, max_days=80)
    qb1 = b.run(10, P[:50], T[:50], S[:50])
    saved = b.get_state()
    c = _model(region, max_days=80)
    c.set_state(saved)
    qc = c.run(60, P[50:], T[50:], S[50:])
    assert np.array_equal(qa, np.concatenate([qb1, qc]))
    for k, v in a.get_state().items():
        assert np.array_equal(v, c.get_state()[k]), k


def test_mass_balance_closes_every_cell():
    from watergap2_gb300 import synthetic as sy
    region = sy.region_small_swb(seed=14)
    P, T, S = sy.forcing(region, 365, doy0=1)
    m = _model(region, max_days=365, record_balance=True)
    s0 = m.balance()[0]
    m.run(1, P, T, S)
    total, pin, evap, out, leak, worst = m.balance()
    resid = (total - s0) - (pin - evap - out + leak)
    assert abs(resid) <= 1e-12 * max(total, pin), (resid, total, pin)
    assert worst <= 1e-12, worst


def test_mass_balance_closes_without_continental_area():
    """Cells whose continental share is below the reference's limit run neither
    the vertical balance nor routing; their inflow leaves the system as a
    negative leak and the balance closes."""
    from watergap2_gb300.region import load_npz
    region, ex = load_npz(os.path.join(os.path.dirname(__file__), "golden", "swb_nocont_150d.npz"))
    P, T, S = ex["P"], ex["T"], ex["S"]
    m = _model(region, max_days=P.shape[0], record_balance=True)
    s0 = m.balance()[0]
    m.run(int(ex["doy0"]), P, T, S)
    total, pin, evap, out, leak, worst = m.balance()
    resid = (total - s0) - (pin - evap - out + leak)
    assert leak < 0.
    assert abs(resid) <= 1e-12 * max(total, pin), (resid, total, pin)
    assert worst <= 1e-12, worst


def test_split_steps_equal_one_launch():
    """A run split into several wg_run_steps calls (wavefront not drained between
    them) equals one wg_run_days call bit for bit."""
    from watergap2_gb300 import synthetic as sy
    region = sy.region_small_swb(seed=15)
    nd = 150
    P, T, S = sy.forcing(region, nd, doy0=250)
    a = _model(region, max_days=nd, stations=np.arange(region.ncell))
    a.upload_forcing(0, P, T, S)
    a.run_days(250, 0, nd)
    b = _model(region, max_days=nd, stations=np.arange(region.ncell))
    b.upload_forcing(0, P, T, S)
    total = b.num_steps(nd)
    cuts = [0, 7, 40, 41, 100, total]
    for t0, t1 in zip(cuts[:-1], cuts[1:]):
        b.run_steps(250, 0, nd, t0, t1)
    assert np.array_equal(a.discharge(0, nd), b.discharge(0, nd))
    for k, v in a.get_state().items():
        assert np.array_equal(v, b.get_state()[k]), k


def test_small_ring_equals_large_ring():
    """The vertical balance run ahead in chunks of a few days gives the same results."""
    from watergap2_gb300 import synthetic as sy
    region = sy.region_64x64(seed=6, size=24)
    P, T, S = sy.forcing(region, 100, doy0=30)
    a = _model(region, max_days=100)
    qa = a.run(30, P, T, S)
    b = _model(region, max_days=100, ring_days=9)
    qb = b.run(30, P, T, S)
    assert np.array_equal(qa, qb)
    for k, v in a.get_state().items():
        assert np.array_equal(v, b.get_state()[k]), k
