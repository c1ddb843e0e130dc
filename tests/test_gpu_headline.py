"""The headline workload end to end on the GPU (libwg_gpu.so through its C ABI).

* The 67,420-cell global grid with every kind of water body, run exactly as
  bench.py runs it -- five days per wavefront step, the default chunks of four
  steps with the next chunk's vertical balance inside the wavefront launches,
  one wg_run_steps call per simulated year, the wavefront never drained between
  years -- against the oracle on the same 5 snow bands over ten simulated years:
  every state field of every cell at the end and the daily discharge of every
  outlet.  (Run with the reference's 100 bands the oracle equals the reference's
  own object code bit for bit on this workload, tests/test_oracle_golden.py; the
  band count changes only the rounding of the band sums.)
* The same launch set-up against the reference's own outputs: the global grid
  over its first 120 days and the 64 x 64 region over a year (fixtures whose
  inputs are regenerated from their seeds).
* Mass balance: the daily closure of the global grid through the per-day entry
  points, and the closure of every cell in the bench's set-up after every
  simulated year.

Tolerance (FP64 path): 1e-10 relative on every field and every station, each
against its own largest value for values below 1e-6 of it (max_rel_err);
closure 1e-12.
"""
import os

import numpy as np
import pytest

from helpers import STATE_KEYS, field_sums, input_digest, max_rel_err, rel_err

pytestmark = pytest.mark.gpu
RTOL = 1e-10
WAVEFRONT_DAYS = 5            # bench.py's days per wavefront step
STEPS_PER_YEAR = 365 // WAVEFRONT_DAYS
YEARS = int(os.environ.get("WG_HEADLINE_YEARS", "10"))


def _station_err(q, qo):
    """Largest max_rel_err over the stations, each on its own scale."""
    return max(max_rel_err(q[:, j], qo[:, j]) for j in range(q.shape[1]))


def _bench_model(region, ndays, **kw):
    from watergap2_gb300.gpu import Model
    return Model(region, max_days=ndays, days_per_step=WAVEFRONT_DAYS, **kw)


def _run_by_year(m, ndays, on_year=None):
    """bench.py's calls: one wg_run_steps per simulated year (the wavefront is
    not drained between them), then the drain."""
    years = ndays // 365
    for y in range(years):
        m.run_steps(1, 0, ndays, y * STEPS_PER_YEAR, (y + 1) * STEPS_PER_YEAR)
        if on_year is not None:
            on_year(y)
    m.run_steps(1, 0, ndays, years * STEPS_PER_YEAR, m.num_steps(ndays))


def test_global_grid_ten_years_as_benchmarked_vs_oracle():
    from oracle import Oracle
    from watergap2_gb300 import synthetic as sy
    region = sy.region_global()
    nd = 365 * YEARS
    P, T, S = sy.forcing_years("region_global", YEARS)
    outlets = np.nonzero(region.downstream < 0)[0]
    m = _bench_model(region, nd, stations=outlets)
    assert m.vertical_overlap() > 0 and m.chunk_steps() == 4      # the bench's launch set-up
    m.upload_forcing(0, P, T, S)
    _run_by_year(m, nd)
    q = m.discharge(0, nd)
    got = m.get_state()
    del m
    o = Oracle(region)
    qo = np.empty_like(q)
    for y in range(YEARS):
        sl = slice(365 * y, 365 * (y + 1))
        qy, _ = o.run(1, P[sl], T[sl], S[sl], discharge=True, nthreads=os.cpu_count() or 1)
        qo[sl] = qy[:, outlets]
    errs = {k: max_rel_err(got[k], o.state[k]) for k in STATE_KEYS + ["snow_band"]}
    errs["discharge"] = _station_err(q, qo)
    print("ten years, largest relative errors:", {k: f"{v:.2e}" for k, v in errs.items() if v > 1e-13})
    assert max(errs.values()) <= RTOL, errs


def _regen(name):
    import importlib.util
    path = os.path.join(os.path.dirname(__file__), "golden", "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", path)
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    ex = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))
    return mg.regen_inputs(name), ex


@pytest.mark.parametrize("name", ["config1_region64_365d", "config2_global_120d"])
def test_gpu_matches_reference_on_workload(name):
    """The reference's own outputs (stations every day, every field of the
    sampled cells, exact sums of every field over all cells) against the GPU
    in the bench's launch set-up, one run per snapshot."""
    (region, P, T, S, doy0, snaps, sample, stations), ex = _regen(name)
    if input_digest(region, P, T, S) != str(ex["digest"]):
        pytest.skip(f"the seeded generators drew different inputs on this host (numpy {np.__version__}); "
                    "the oracle tests cover this workload")
    keys = [str(k) for k in ex["keys"]]
    m = _bench_model(region, P.shape[0], stations=stations)
    m.upload_forcing(0, P, T, S)
    day, doy = 0, doy0
    for i, sd in enumerate(snaps):
        m.run_days(doy, day, sd - day)
        doy = (doy - 1 + (sd - day)) % 365 + 1
        day = sd
        st = m.get_state()
        st["snow_band"] = st["snow_band"].reshape(region.ncell, region.nband)
        sums = field_sums(st, keys + ["snow_band"])
        assert rel_err(sums, ex[f"s{i}_sums"]) <= RTOL, (i, sums, ex[f"s{i}_sums"])
        if f"s{i}_soil" in ex:
            errs = {k: max_rel_err(st[k][sample], ex[f"s{i}_{k}"]) for k in keys + ["snow_band"]}
            res = region.res_area[sample] > 0
            errs["k_release"] = max_rel_err(st["k_release"][sample][res], ex[f"s{i}_k_release"][res])
            assert max(errs.values()) <= RTOL, errs
    assert _station_err(m.discharge(0, P.shape[0]), ex["discharge"]) <= RTOL


def test_global_grid_daily_closure_per_day_entry_points():
    """Every day of a year on the global grid: the change of the total storage
    equals inflow - evaporation - outflow + clamp corrections of that day, and
    every cell's own balance closes, both to 1e-12 of the day's throughput."""
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_global()
    nd = 365
    P, T, S = sy.forcing(region, nd, seed=2, doy0=1)
    m = Model(region, max_days=nd, record_balance=True)
    m.upload_forcing(0, P, T, S)
    prev = m.balance()
    worst_day, worst_cell = 0.0, 0.0
    for d in range(nd):
        m.step_vertical(d + 1, d)
        m.step_routing(d + 1, d)
        b = m.balance()
        dS = b[0] - prev[0]
        flux = (b[1] - prev[1]) - (b[2] - prev[2]) - (b[3] - prev[3]) + (b[4] - prev[4])
        thru = max(b[1] - prev[1], b[2] - prev[2], b[3] - prev[3])
        worst_day = max(worst_day, abs(dS - flux) / thru)
        worst_cell = max(worst_cell, b[5])
        prev = b
    assert worst_day <= 1e-12 and worst_cell <= 1e-12, (worst_day, worst_cell)


def test_global_grid_closure_every_year_as_benchmarked():
    """The bench's launch set-up with the balance recorded: after every yearly
    call (cells on different days in the wavefront) every cell's balance closes,
    and after the drain the global balance closes; two years."""
    from watergap2_gb300 import synthetic as sy
    region = sy.region_global()
    nd = 730
    P, T, S = sy.forcing(region, nd, seed=2, doy0=1)
    m = _bench_model(region, nd, record_balance=True)
    m.upload_forcing(0, P, T, S)
    s0 = m.balance()[0]
    cells = []
    _run_by_year(m, nd, on_year=lambda y: cells.append(m.balance()[5]))
    total, pin, evap, out, leak, worst = m.balance()
    resid = (total - s0) - (pin - evap - out + leak)
    assert abs(resid) <= 1e-12 * max(total, pin), (resid, total, pin)
    assert max(cells) <= 1e-12 and worst <= 1e-12, (cells, worst)
