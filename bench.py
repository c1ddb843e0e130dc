"""Benchmark of the WaterGAP2 daily step on GB300 (cell-days/s).

Workload (the largest single-GPU configuration the metric is quoted on): the
plain FP64 global 0.5-degree grid, 67,420 land cells with local lakes,
wetlands, 300 global lakes and 1,200 reservoirs, D8 drainage with ~6,000
outlets; seeded synthetic inputs (no dataset).  One step = one simulated year
(365 days) of the whole grid, i.e. 24.6 M cell-days; the default 10 timed
steps are the 10-year run (246.1 M cell-days).

  value  device-resident: forcing for all years is in HBM before timing; each
         step is one persistent launch of the day-pipelined kernel (wg_run_days).
  e2e    through the C ABI with host buffers: every step copies that year's
         forcing from pinned host memory (wg_upload_forcing) and reads the
         outlet discharge back (wg_get_discharge).
  --impl reference  the reference's CPU algorithm (the oracle port of
         daily.cpp/routing.cpp) on the host cores, same metric.

Run:  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-days/s on 1 GB300 (plain FP64 vs batched FP32 ensemble) at stated error"
DAYS_PER_STEP = 365
# days every cell advances per wavefront step (wg_options.days_per_step): the
# step barrier and the start-of-step load latency are paid once per 5 days; a
# timed step (one year) is 73 wavefront steps.  Results are the same bits.
WAVEFRONT_DAYS = 5
WSTEPS_PER_YEAR = DAYS_PER_STEP // WAVEFRONT_DAYS
# algorithmic HBM bytes per cell-day of a day-by-day FP64 implementation with the
# water bodies of this workload: vertical 224 + routing 96 + water bodies ~4
BYTES_PER_CELL_DAY = 324.0
# of which the routing part of the wavefront kernel k_pipeline moves: routing 96 +
# water bodies 4 + the vertical balance of the cells with water bodies (7.2 % of
# the cells x 224)
WAVEFRONT_BYTES_PER_CELL_DAY = 116.2
# the vertical balance of one cell-day without water bodies (run ahead of routing:
# by k_vertical_ahead, or by the extra warps of the wavefront launches)
VERTICAL_BYTES_PER_CELL_DAY = 224.0


def profile_figures(path=os.path.join(ROOT, "profiles", "fp64_global_wavefront_kernels.md")):
    """The '- name kernel: value' lines of the committed ncu summary."""
    out = {}
    if os.path.exists(path):
        for line in open(path):
            line = line.strip()
            if line.startswith("- ") and ":" in line:
                k, v = line[2:].rsplit(":", 1)
                try:
                    out[k.strip()] = float(v)
                except ValueError:
                    pass
    return out


def make_forcing(nyears, seed=2, procs=None):
    """Forcing for nyears years of the global grid, one year per spawned worker
    (before any CUDA context exists)."""
    from watergap2_gb300 import synthetic as sy
    return sy.forcing_years("region_global", nyears, seed=seed, procs=procs)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            out, _ = self.proc.communicate(timeout=10)
            self.lines = [l for l in out.splitlines() if l.strip()]
        return False

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_sample(region, ndays, threads):
    """The oracle port over ndays of the workload; returns (cell-days/s, seconds)."""
    from oracle import Oracle
    from watergap2_gb300 import synthetic as sy
    P, T, S = sy.forcing(region, ndays, seed=2, doy0=1)
    o = Oracle(region)
    t0 = time.perf_counter()
    o.run(1, P, T, S, nthreads=threads)
    dt = time.perf_counter() - t0
    return region.ncell * ndays / dt, dt


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU algorithm on the host cores.  Each
    step is one simulated year (365 days) of the global grid, run by the oracle
    port (vertical pass on every host thread, routing serial), the state carried
    from step to step as in a multi-year run; warm-up steps are the same years
    untimed.  The forcing (one year, reused every year) is generated before the
    steps."""
    if rank != 0:
        return
    from oracle import Oracle
    from watergap2_gb300 import synthetic as sy
    region = sy.region_global()
    threads = os.cpu_count() or 1
    days = int(os.environ.get("WG_REF_STEP_DAYS", str(DAYS_PER_STEP)))
    P, T, S = sy.forcing(region, days, seed=2, doy0=1)
    o = Oracle(region)
    for _ in range(args.warmup):
        o.run(1, P, T, S, nthreads=threads)
    secs = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.run(1, P, T, S, nthreads=threads)
        secs.append(time.perf_counter() - t0)
    total = sum(secs)
    value = region.ncell * days * args.steps / total
    split = Oracle.last_timing()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cell-days/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generators)",
        "config": {"workload": "global 0.5-degree grid, 67,420 cells, lakes/wetlands/reservoirs, FP64, "
                               f"1 step = {days} days of every cell",
                   "ncell": region.ncell, "days_per_timed_step": days},
        "cpu_baseline": {"value": value, "unit": "cell-days/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} steps of {days} days x {region.ncell} cells, vertical pass on "
                                   f"{threads} OpenMP threads, routing serial as in the reference; last step "
                                   f"vertical {split['vertical_s']:.2f} s, routing {split['routing_s']:.2f} s"},
        "e2e": {"value": value, "unit": "cell-days/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


ENS_MEMBERS = 256
ENS_DAYS = 730


def outlet_errors(q_test, q_ref):
    """Per-outlet discharge error of q_test against q_ref ([days, outlets]):
    mean error |mean q - mean ref| / mean ref, and daily error max |q - ref| over
    the days relative to the outlet's peak reference discharge."""
    scale = np.maximum(np.abs(q_ref).max(axis=0), 1e-30)
    daily = np.abs(q_test - q_ref).max(axis=0) / scale
    mean = np.abs(q_test.mean(axis=0) - q_ref.mean(axis=0)) / np.maximum(np.abs(q_ref.mean(axis=0)), 1e-30)
    return {"mean_err_max": float(mean.max()), "daily_err_median": float(np.median(daily)),
            "daily_err_q99": float(np.quantile(daily, 0.99)), "daily_err_max": float(daily.max())}


def run_water_temp(region, P, T, S, stream, local):
    """The global grid with the water temperature (wg_options.water_temp: the
    reference's calcWTemp for the river and every water body after each cell's
    routing, with fractional routing) against the plain run: four years in one
    wavefront, the fourth timed with CUDA events (the first three fill the
    wavefront: 219 steps of 5 days for its 198 levels)."""
    import torch
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    nd = 4 * DAYS_PER_STEP
    LW, GWT = sy.water_temp_inputs(region, nd, T[:nd])
    out = {}
    # as the reference's option parser does, the water temperature runs with
    # fractional routing (option.cpp:591-593)
    region_wt = region.with_options(frac_routing=1)
    for name, kw in (("water_temp", dict(water_temp=True)), ("without", dict()),
                     ("without_overlap_off", dict())):   # the vertical overlap is on in the first two
        m = Model(region_wt if kw else region, max_days=nd, device=local, stream=stream.cuda_stream,
                  days_per_step=WAVEFRONT_DAYS, **kw)
        if name == "without_overlap_off":
            m.vertical_overlap(False)
        m.upload_forcing(0, P[:nd], T[:nd], S[:nd])
        if kw:
            m.set_water_temp_inputs(GWT)
            m.upload_longwave(0, LW)
        assert 3 * WSTEPS_PER_YEAR >= m.num_levels - 1
        m.run_steps(1, 0, nd, 0, 3 * WSTEPS_PER_YEAR)
        m.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        m.run_steps(1, 0, nd, 3 * WSTEPS_PER_YEAR, 4 * WSTEPS_PER_YEAR)
        e1.record(stream)
        m.synchronize()
        ms = e0.elapsed_time(e1)
        out[name] = {"cell_days_per_s": region.ncell * DAYS_PER_STEP / (ms / 1000.0), "ms_per_year": ms}
        if kw:
            t, ice = m.water_temp()
            out[name]["river_temp_mean"] = float(np.mean(t[0]))
            out[name]["cells_with_river_ice"] = int(np.sum(ice[0] > 0))
        del m
    out["cost_vs_plain"] = out["without"]["cell_days_per_s"] / out["water_temp"]["cell_days_per_s"]
    # the oracle port with the water temperature on the host cores (a bounded sample)
    from oracle import Oracle
    cpu_days = int(os.environ.get("WG_CPU_WT_SAMPLE_DAYS", "200"))
    threads = os.cpu_count() or 1
    o = Oracle(region_wt)
    o.init_water_temp(GWT)
    t0 = time.perf_counter()
    o.run_wt(1, P[:cpu_days], T[:cpu_days], S[:cpu_days], LW[:cpu_days], nthreads=threads)
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": region.ncell * cpu_days / cpu_s, "unit": "cell-days/s", "cores": threads,
                           "kind": "port", "sample": f"{cpu_days} days of the same grid ({cpu_s:.1f} s)"}
    return out


def run_water_use(region, P, T, S, stream, local):
    """The global grid with water use (wg_options.water_use: the reference's
    subtract_use = 2, every cell meeting its monthly net abstractions from its own
    global lake, reservoir, river, local lake and groundwater) against the plain
    run: four years in one wavefront with each year's tables, the fourth timed
    with CUDA events (the first three fill the wavefront).  Synthetic monthly net
    abstractions (synthetic.water_use_inputs, seeded).  The "glwd" leg adds the
    GLWD units of synthetic.glwd_units (aggrNUsGloLakResOpt = 1: the riparian
    cells' use met by their global lake's or reservoir's outflow cell; each
    unit's cells routed by one thread)."""
    import torch
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    nd = 4 * DAYS_PER_STEP
    nus, nug, wdr, cons, frgi = sy.water_use_inputs(region, 4)
    use = (nus, nug, wdr, cons)
    out = {}
    unit = sy.glwd_units(region)
    for name, kw in (("water_use", dict(water_use=True)), ("glwd", dict(water_use=True, glwd_unit=unit)),
                     ("without", dict())):
        m = Model(region, max_days=nd, device=local, stream=stream.cuda_stream, days_per_step=WAVEFRONT_DAYS, **kw)
        m.upload_forcing(0, P[:nd], T[:nd], S[:nd])
        if kw:
            m.set_water_use_inputs(frgi)
            m.upload_water_use_run(0, 1, nd, use)
        assert 3 * WSTEPS_PER_YEAR >= m.num_levels - 1
        m.run_steps(1, 0, nd, 0, 3 * WSTEPS_PER_YEAR)
        m.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        m.run_steps(1, 0, nd, 3 * WSTEPS_PER_YEAR, 4 * WSTEPS_PER_YEAR)
        e1.record(stream)
        m.synchronize()
        ms = e0.elapsed_time(e1)
        out[name] = {"cell_days_per_s": region.ncell * DAYS_PER_STEP / (ms / 1000.0), "ms_per_year": ms}
        if kw:
            w = m.water_use()
            out[name]["actual_use_km3_last_year"] = float(np.sum(w[11]))
            out[name]["unsatisfied_km3_last_year"] = float(np.sum(w[6]))
        if "glwd_unit" in kw:
            out[name]["glwd_units"] = int(unit.max())
            out[name]["cells_in_units"] = int((unit > 0).sum())
            out[name]["levels"] = m.num_levels
        del m
    out["cost_vs_plain"] = out["without"]["cell_days_per_s"] / out["water_use"]["cell_days_per_s"]
    out["glwd_cost_vs_water_use"] = out["water_use"]["cell_days_per_s"] / out["glwd"]["cell_days_per_s"]
    # the oracle port with water use on the host cores (a bounded sample)
    from oracle import Oracle
    cpu_days = int(os.environ.get("WG_CPU_WU_SAMPLE_DAYS", "200"))
    threads = os.cpu_count() or 1
    o = Oracle(region)
    o.init_water_use(frgi)
    t0 = time.perf_counter()
    o.run_wu(1, P[:cpu_days], T[:cpu_days], S[:cpu_days], use, nthreads=threads)
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": region.ncell * cpu_days / cpu_s, "unit": "cell-days/s", "cores": threads,
                           "kind": "port", "sample": f"{cpu_days} days of the same grid ({cpu_s:.1f} s)"}
    return out


def run_outputs(region, P, T, S, stream, local):
    """The global grid with the output grids against the plain run: routing's
    monthly aggregates only (wg_monthly_outputs: river availability with its
    minimum and maximum, cell runoff, velocity, storage); with the vertical
    balance's 33 monthly grids (wg_monthly_outputs_vertical; the reference's
    grid_store = 2 sums); with routing's further 10 monthly grids as well
    (wg_monthly_outputs_routing); and with every daily grid too (27 of the
    vertical balance, 9 of routing, kept on the device for all four years:
    grid_store = 6).  Four years in one wavefront, the fourth timed with CUDA
    events (the first three fill the wavefront)."""
    import torch
    from watergap2_gb300.gpu import Model
    nd = 4 * DAYS_PER_STEP
    out = {}
    # grids: 1 routing's monthly aggregates, 2 and the vertical balance's monthly
    # grids, 3 and routing's further monthly grids, 4 all of them and every daily
    # grid (vertical balance and routing) for the four years
    for name, grids in (("routing_grids", 1), ("all_grids", 2), ("all_monthly_grids", 3),
                        ("monthly_and_daily_grids", 4), ("without", 0)):
        m = Model(region, max_days=nd, device=local, stream=stream.cuda_stream, days_per_step=WAVEFRONT_DAYS)
        if grids:
            m.monthly_outputs(48, doy_day0=1)
            m.monthly_outputs_vertical(grids >= 2)
            m.monthly_outputs_routing(grids >= 3)
        if grids == 4:
            m.daily_outputs_vertical(nd)
            m.daily_outputs_routing(nd)
        m.upload_forcing(0, P[:nd], T[:nd], S[:nd])
        assert 3 * WSTEPS_PER_YEAR >= m.num_levels - 1
        m.run_steps(1, 0, nd, 0, 3 * WSTEPS_PER_YEAR)
        m.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        m.run_steps(1, 0, nd, 3 * WSTEPS_PER_YEAR, 4 * WSTEPS_PER_YEAR)
        e1.record(stream)
        m.synchronize()
        ms = e0.elapsed_time(e1)
        out[name] = {"cell_days_per_s": region.ncell * DAYS_PER_STEP / (ms / 1000.0), "ms_per_year": ms}
        if grids == 2:   # a sanity figure: the first year's mean monthly precipitation sum [mm]
            # (every cell has finished the first year; the wavefront's upstream
            # cells have not finished the fourth when the timed steps end)
            out[name]["mean_monthly_prec_mm"] = float(np.mean(m.monthly("prec", 0, 12)))
        del m
    for name in ("routing_grids", "all_grids", "all_monthly_grids", "monthly_and_daily_grids"):
        out[name]["cost_vs_plain"] = out["without"]["cell_days_per_s"] / out[name]["cell_days_per_s"]
    return out


# algorithmic HBM bytes per member-cell-day of the ensemble (FP32 state, the
# forcing and static parameters shared by the members of one cell in a block):
# per member state r+w 72, perturbed gamma 4, outputs 8; per block of members
# forcing 12 + static parameters 40
ENS_BYTES_PER_MEMBER = 84.0
ENS_BYTES_PER_BLOCK = 52.0


def ensemble_member_errors(region, P, T, S, pf, gf, ens, nd, stream, local):
    """Discharge error of every member of the ensemble against an FP64 run of the
    same member's inputs (precipitation x pf[m], gamma x gf[m]): per member the
    outlet errors of outlet_errors; summarised over the members."""
    from watergap2_gb300.gpu import Model
    ref = Model(region, max_days=nd, device=local, stream=stream.cuda_stream, days_per_step=WAVEFRONT_DAYS,
                stations=ens.stations)
    ref.upload_forcing(0, P, T, S)
    ref.save_snapshot()
    g0 = region.param("P_GAMRUN_C").copy()
    rows = []
    for m in range(ens.members):
        ref.restore_snapshot()
        ref.set_calib_param("P_GAMRUN_C", g0 * float(gf[m]))
        ref.upload_forcing(0, (P * pf[m]).astype(np.float32), None, None)
        ref.run_days(1, 0, nd)
        rows.append(outlet_errors(ens.member_discharge(m, 0, nd), ref.discharge(0, nd)))
    del ref
    keys = rows[0].keys()
    arr = {k: np.array([r[k] for r in rows]) for k in keys}
    return {"members": len(rows),
            "daily_err_max": {"max": float(arr["daily_err_max"].max()),
                              "median": float(np.median(arr["daily_err_max"])),
                              "q99": float(np.quantile(arr["daily_err_max"], 0.99)),
                              "members_above_1e-5": int((arr["daily_err_max"] > 1e-5).sum())},
            "mean_err_max": {"max": float(arr["mean_err_max"].max()),
                             "median": float(np.median(arr["mean_err_max"]))},
            "daily_err_q99_max": float(arr["daily_err_q99"].max()),
            "member0": rows[0], "worst_member": int(np.argmax(arr["daily_err_max"]))}


def run_ensemble(args, region, P, T, S, stream, local, plain_value):
    """Batched ensemble: ENS_MEMBERS members of the global grid over ENS_DAYS days in
    one day-pipelined wavefront (FP32 state, FP64 confluence and balance sums),
    launch shape and chunk length from the autotuner, the whole run captured in one
    CUDA graph and replayed.  Members: precipitation x lognormal(0, 0.3), runoff
    coefficient gamma x U(0.7, 1.3), each from its own seed; member 0 unperturbed.
    Discharge error: every member of the first replay against an FP64 run of its
    own inputs."""
    import torch
    from watergap2_gb300.gpu import Model
    M, nd = ENS_MEMBERS, ENS_DAYS
    P, T, S = P[:nd], T[:nd], S[:nd]
    pf = np.array([np.exp(np.random.default_rng((7, m)).normal(0.0, 0.3)) for m in range(M)], np.float32)
    gf = np.array([np.random.default_rng((8, m)).uniform(0.7, 1.3) for m in range(M)], np.float32)
    pf[0] = gf[0] = 1.0
    ens = Model(region, max_days=nd, device=local, stream=stream.cuda_stream, precision="fp32", members=M,
                prec_factor=pf, gamma_factor=gf, days_per_step=WAVEFRONT_DAYS)
    ens.upload_forcing(0, P, T, S)
    total = ens.num_steps(nd)
    lag = ens.num_levels - 1
    tune = ens.autotune(1, 0, nd, lag, 64)
    ens.graph_capture(1, 0, nd, 0, total)
    # first replay: from the initial state, checked against FP64
    ens.graph_launch()
    ens.synchronize()
    errors = ensemble_member_errors(region, P, T, S, pf, gf, ens, nd, stream, local)
    for _ in range(max(0, args.warmup - 1)):
        ens.graph_launch()
    ens.synchronize()
    l0 = ens.launch_count
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    reps = max(1, min(args.steps, 3))
    for _ in range(reps):
        ens.graph_launch()
    e1.record(stream)
    torch.cuda.synchronize()
    ens.synchronize()
    ms = e0.elapsed_time(e1) / reps
    value = M * region.ncell * nd / (ms / 1000.0)
    # roofline of the whole run (both kernels of each launch pair move the
    # algorithmic bytes counted per member-cell-day; the run is one CUDA graph)
    peaks, peak_kind = measured_peaks()
    per_mcd = ENS_BYTES_PER_MEMBER + ENS_BYTES_PER_BLOCK / tune["threads"]
    achieved = value * per_mcd / 1e9
    figs = profile_figures(os.path.join(ROOT, "profiles", "ensemble_global_kernels.md"))
    traffic = figs.get("dram_bytes_per_member_cell_day")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                "frac": achieved / peaks.get("hbm_gbs"), "peak_kind": peak_kind,
                "algorithmic_bytes_per_member_cell_day": per_mcd,
                "traffic_bytes_per_member_cell_day": traffic,
                "kernel": "k_vertical_ahead<float,1> + k_pipeline<float,1,1> (whole graph-captured run)"}
    return {"metric": "member-cell-days/s", "value": value, "members": M, "days": nd, "ncell": region.ncell,
            "ms_per_run": ms, "runs_timed": reps, "gpu_launches": int(ens.launch_count - l0),
            "dtype": "f32 state, f64 sums", "vs_plain_fp64": value / plain_value, "autotune": tune,
            "graph": "whole run (all launch pairs) captured once, replayed per run",
            "roofline": roofline, "discharge_error_vs_fp64": errors}


def run_closure(region, P, T, S, stream, local, ndays=365):
    """The daily mass-balance closure of the global grid (FP64, compensated sums):
    one year through the per-day entry points with the balance recorded; each
    day the change of the total storage against that day's inflow - evaporation
    - outflow + clamp corrections, relative to the day's throughput, and the
    largest per-cell closure residual."""
    from watergap2_gb300.gpu import Model
    m = Model(region, max_days=ndays, device=local, stream=stream.cuda_stream, record_balance=True)
    m.upload_forcing(0, P[:ndays], T[:ndays], S[:ndays])
    prev = m.balance()
    daily, cells = [], []
    for d in range(ndays):
        m.step_vertical(d + 1, d)
        m.step_routing(d + 1, d)
        b = m.balance()
        flux = (b[1] - prev[1]) - (b[2] - prev[2]) - (b[3] - prev[3]) + (b[4] - prev[4])
        daily.append(abs((b[0] - prev[0]) - flux) / max(b[1] - prev[1], b[2] - prev[2], b[3] - prev[3]))
        cells.append(b[5])
        prev = b
    del m
    return {"days": ndays, "max_daily_residual_rel": float(max(daily)),
            "median_daily_residual_rel": float(statistics.median(daily)),
            "max_cell_residual_rel": float(max(cells)), "bound": 1e-12,
            "closed_every_day": bool(max(daily) <= 1e-12 and max(cells) <= 1e-12)}


def fp64_peak_tflops():
    from watergap2_gb300 import gpu
    return gpu.measure_fp64_peak()


def run_gpu(args, rank, world):
    import torch
    from watergap2_gb300 import replicas
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    region = sy.region_global()
    nyears = args.warmup + args.steps
    P, T, S = args.forcing
    stream = torch.cuda.Stream(device=local)
    model = Model(region, max_days=nyears * DAYS_PER_STEP, device=local, stream=stream.cuda_stream,
                  days_per_step=WAVEFRONT_DAYS)
    nst = model.stations.size

    # ---- value: device-resident forcing.  The whole nyears-year run is one
    # day-pipelined wavefront; each step is one call covering 365 wavefront steps,
    # so after the warm-up every timed call routes exactly 365 days of every cell.
    ndays = nyears * DAYS_PER_STEP
    model.upload_forcing(0, P, T, S)
    model.synchronize()
    total_steps = model.num_steps(ndays)
    assert args.warmup * WSTEPS_PER_YEAR >= model.num_levels - 1, "warm-up must fill the wavefront"
    model.run_steps(1, 0, ndays, 0, args.warmup * WSTEPS_PER_YEAR)
    model.synchronize()
    launches0 = model.launch_count
    model.kernel_timing(True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    per_step = []
    with ClockSampler(local) as clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        for k in range(args.steps):
            t0 = (args.warmup + k) * WSTEPS_PER_YEAR
            e_a, e_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e_a.record(stream)
            model.run_steps(1, 0, ndays, t0, t0 + WSTEPS_PER_YEAR)
            e_b.record(stream)
            per_step.append((e_a, e_b))
        ev1.record(stream)
        torch.cuda.synchronize()
        model.synchronize()
        if dist:
            dist.barrier()
    gpu_launches = model.launch_count - launches0
    kernel_ms = model.kernel_times()
    model.kernel_timing(False)
    vinline_frac = model.vinline_fraction()
    chunk_steps, overlap_warps = model.chunk_steps(), model.vertical_overlap()
    elapsed_ms = ev0.elapsed_time(ev1)
    launch_ms = [a.elapsed_time(b) for a, b in per_step]
    model.run_steps(1, 0, ndays, nyears * WSTEPS_PER_YEAR, total_steps)   # drain (untimed)
    model.synchronize()
    elapsed_ms = replicas.job_seconds(elapsed_ms / 1000.0, dist, device="cuda") * 1000.0   # max over ranks
    cell_days = region.ncell * DAYS_PER_STEP * args.steps
    value = replicas.whole_job_value(cell_days, world, elapsed_ms / 1000.0)
    lag = (model.num_levels - 1) * WAVEFRONT_DAYS   # days a cell trails the first cells
    q_dev = model.discharge(0, ndays)

    # ---- e2e: the same run through the C ABI with host buffers: every step copies
    # that year's forcing from pinned host memory and reads back the outlet
    # discharge of the 365 days the step completed
    del model
    e2e_model = Model(region, max_days=ndays + DAYS_PER_STEP, device=local, stream=stream.cuda_stream,
                      days_per_step=WAVEFRONT_DAYS)
    pin = [torch.empty((ndays, region.ncell), dtype=torch.float32, pin_memory=True) for _ in range(3)]
    for t_, a in zip(pin, (P, T, S)):
        t_.numpy()[:] = a
    Pn, Tn, Sn = (t_.numpy() for t_ in pin)
    hostq = torch.empty((DAYS_PER_STEP, nst), dtype=torch.float64, pin_memory=True).numpy()

    phases = []   # per timed step: CUDA-event ms of the run, host ms of the whole step

    def upload(k, overlap):
        # year k into day slots of year k; the step after the last year uploads year 0's
        # data into a spare year of slots, so every step moves one year of forcing
        src = (k % nyears) * DAYS_PER_STEP
        sl = slice(src, src + DAYS_PER_STEP)
        e2e_model.upload_forcing(k * DAYS_PER_STEP, Pn[sl], Tn[sl], Sn[sl], overlap=overlap)

    def e2e_step(k, record=False):
        # year k's forcing is on the device (uploaded during step k-1); this step
        # runs year k, uploads year k+1 on the copy stream alongside the run, and
        # reads back the discharge of the days the step completed
        h0 = time.perf_counter()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)] if record else None
        if record:
            ev[0].record(stream)
        e2e_model.run_steps(1, 0, ndays, k * WSTEPS_PER_YEAR, (k + 1) * WSTEPS_PER_YEAR)
        if record:
            ev[1].record(stream)
        upload(k + 1, overlap=True)
        d0 = max(0, (k + 1) * DAYS_PER_STEP - lag - DAYS_PER_STEP)
        e2e_model.discharge_into(d0, DAYS_PER_STEP, hostq)   # synchronises the run
        if record:
            phases.append((ev[0].elapsed_time(ev[1]), 1e3 * (time.perf_counter() - h0)))

    upload(0, overlap=False)

    for w in range(args.warmup):
        e2e_step(w)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(args.warmup + k, record=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_model.run_steps(1, 0, ndays, nyears * WSTEPS_PER_YEAR, total_steps)
    same = bool(np.array_equal(e2e_model.discharge(0, ndays), q_dev))
    e2e_s = replicas.job_seconds(e2e_s, dist, device="cuda")
    e2e_value = replicas.whole_job_value(cell_days, world, e2e_s)
    h2d = 3 * DAYS_PER_STEP * region.ncell * 4
    d2h = DAYS_PER_STEP * nst * 8
    num_levels = e2e_model.num_levels

    del e2e_model
    # the reference's granularity through the C ABI: per day one whole-grid
    # calcNewDay call and one routing call (integrate_wghm_'s loop, which the C++
    # stand-ins of include/wg_gpu.hpp keep), the model read at every month end:
    # with the calls deferred (wg_set_deferred, the stand-ins' mode) each month
    # runs as one day-pipelined launch sequence; immediate: two launches a day
    per_day = None
    if rank == 0:
        per_day = {"api": "wg_step_vertical + wg_step_routing per day, state read at every month end "
                          "(integrate_wghm_'s loop through the drop-in stand-ins)"}
        month_end = set(np.cumsum([31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31]).tolist())
        for name, deferred, nd in (("deferred", True, DAYS_PER_STEP), ("immediate", False, 60)):
            pd = Model(region, max_days=nd, device=local, stream=stream.cuda_stream)
            pd.upload_forcing(0, P[:nd], T[:nd], S[:nd])
            pd.synchronize()
            if deferred:
                pd.set_deferred(True)
            t0 = time.perf_counter()
            for d in range(nd):
                pd.step_vertical(d + 1, d)
                pd.step_routing(d + 1, d)
                if d + 1 in month_end:   # what integrate_wghm_ reads at a month end (integrateWGHM.cpp:830-847)
                    pd.get_state(fields=("canopy", "soil", "snow", "snow_band", "laf"))
            pd.synchronize()
            sec = time.perf_counter() - t0
            per_day[name] = {"value": region.ncell * nd / sec, "unit": "cell-days/s", "days": nd,
                             "ms_per_day": 1000.0 * sec / nd}
            del pd
        per_day["value"] = per_day["deferred"]["value"]
        per_day["unit"] = "cell-days/s"
    closure = run_closure(region, P, T, S, stream, local) if rank == 0 else None
    ensemble = None
    if rank == 0 and not os.environ.get("WG_BENCH_NO_ENSEMBLE"):
        ensemble = run_ensemble(args, region, P, T, S, stream, local, value)
    water_temp = None
    if rank == 0 and not os.environ.get("WG_BENCH_NO_WTEMP"):
        water_temp = run_water_temp(region, P, T, S, stream, local)
    water_use = None
    if rank == 0 and not os.environ.get("WG_BENCH_NO_WUSE"):
        water_use = run_water_use(region, P, T, S, stream, local)
    outputs = None
    if rank == 0 and not os.environ.get("WG_BENCH_NO_OUTPUTS"):
        outputs = run_outputs(region, P, T, S, stream, local)
    # the other configurations, bounded: one simulated year of the 5-arc-minute
    # grid in both precisions, and the learned-calibration workload
    fine = None
    if rank == 0 and not os.environ.get("WG_BENCH_NO_FINE"):
        fine = fine_workload(1, device=local)
    calibration = None
    if rank == 0 and not os.environ.get("WG_BENCH_NO_CALIB"):
        calibration = calibration_workload(device=local)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peaks, peak_kind = measured_peaks()
    # dominant kernel: the wavefront kernel k_pipeline, its device time from the CUDA
    # events the library records around each launch.  Each timed step (one call of
    # 365 wavefront steps) is one k_vertical_ahead launch for the first chunk and
    # ceil(365 / chunk) wavefront launches, all but the last carrying the vertical
    # balance of the next chunk's cells without water bodies (with the overlap on;
    # without it, one k_vertical_ahead launch before every wavefront launch).
    n_wave = kernel_ms["launch_pairs"]
    pipe_ms_total, va_ms_total = kernel_ms["wavefront_ms"], kernel_ms["vertical_ahead_ms"]
    pipe_ms = pipe_ms_total / n_wave
    nplain = region.ncell * (1.0 - vinline_frac)
    route_cd = region.ncell * DAYS_PER_STEP * args.steps                 # routing cell-days
    va_days = chunk_steps * WAVEFRONT_DAYS if overlap_warps else DAYS_PER_STEP
    va_alone_cd = nplain * va_days * args.steps                         # k_vertical_ahead
    va_wave_cd = nplain * (DAYS_PER_STEP - va_days) * args.steps        # extra warps of k_pipeline
    wave_bytes = WAVEFRONT_BYTES_PER_CELL_DAY * route_cd + VERTICAL_BYTES_PER_CELL_DAY * va_wave_cd
    achieved = wave_bytes / (pipe_ms_total / 1000.0) / 1e9
    figs = profile_figures()
    traffic = None
    if overlap_warps and chunk_steps == figs.get("chunk_steps") and WAVEFRONT_DAYS == figs.get("days_per_step"):
        traffic = figs.get("traffic_bytes_per_launch k_pipeline")       # a launch of the same shape
    fp64 = None
    try:
        peak64 = fp64_peak_tflops()
        fp64 = {"peak": peak64, "unit": "TFLOP/s", "peak_kind": "measured (DFMA loop)"}
        fl_route = figs.get("fp64_flops_per_cell_day routing")
        fl_va = figs.get("fp64_flops_per_cell_day k_vertical_ahead")
        if fl_route is not None and fl_va is not None:
            for kname, ms, flops in (("k_pipeline", pipe_ms_total, fl_route * route_cd + fl_va * va_wave_cd),
                                     ("k_vertical_ahead", va_ms_total, fl_va * va_alone_cd)):
                ach = flops / (ms / 1000.0) / 1e12
                fp64[kname] = {"achieved": ach, "frac": ach / peak64, "ms_per_timed_step": ms / args.steps,
                               "pipe_busy_ncu": figs.get(f"fp64_pipe_busy {kname}")}
            fp64["flops_per_cell_day"] = {"routing": fl_route, "vertical": fl_va}
    except Exception as exc:   # diagnostics only
        fp64 = {"error": str(exc)}
    cpu_threads = os.cpu_count() or 1
    cpu_days = int(os.environ.get("WG_CPU_SAMPLE_DAYS", "1000"))
    cpu_val, cpu_s = cpu_sample(region, cpu_days, cpu_threads)
    line = {
        "metric": METRIC, "value": value, "unit": "cell-days/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generators)",
        "config": {"workload": "global 0.5-degree grid, 67,420 cells, lakes/wetlands/reservoirs, FP64, "
                               "1 step = 365 days of every cell (10 steps = the 10-year run)",
                   "ncell": region.ncell, "days_per_timed_step": DAYS_PER_STEP,
                   "days_per_wavefront_step": WAVEFRONT_DAYS, "levels": num_levels,
                   "stations": int(nst), "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (295 MB of forcing read per step)"},
        "gpu_launches": int(gpu_launches),
        "e2e": {"value": e2e_value, "unit": "cell-days/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "matches_device_run": same,
                "phases_ms": {"run": statistics.mean(p[0] for p in phases),
                              "step_host": statistics.mean(p[1] for p in phases)},
                "upload": "next year's forcing on the copy stream, overlapped with this year's run"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": achieved / peaks.get("hbm_gbs"), "traffic": traffic,
                     "peak_kind": peak_kind,
                     "kernel": f"k_pipeline (wavefront, {chunk_steps} steps per launch, "
                               f"{overlap_warps} vertical-balance warps per block)",
                     "algorithmic_bytes_per_cell_day": {"routing": WAVEFRONT_BYTES_PER_CELL_DAY,
                                                        "vertical": VERTICAL_BYTES_PER_CELL_DAY},
                     "launch_ms": pipe_ms, "launches_per_timed_step": n_wave / args.steps,
                     "limiter": "FP64 pipe (see fp64), not HBM",
                     "vertical_ahead_ms_per_timed_step": va_ms_total / args.steps},
        "fp64": fp64,
        "per_day_api": per_day,
        "closure": closure,
        "ensemble": ensemble,
        "water_temp": water_temp,
        "water_use": water_use,
        "outputs": outputs,
        "fine_5min": fine,
        "calibration": calibration,
        "cpu_baseline": {"value": cpu_val, "unit": "cell-days/s", "cores": cpu_threads, "kind": "port",
                         "sample": f"{cpu_days} days of the same grid ({region.ncell * cpu_days} cell-days, "
                                   f"{cpu_s:.1f} s), vertical pass on {cpu_threads} OpenMP threads, routing serial"},
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_profile_case(steps: int = 24, warm_steps: int = 200, outputs: bool = False):
    """A short, self-contained case for ncu: the global grid as the bench runs it
    (WAVEFRONT_DAYS days per wavefront step, default chunks of 4 steps, vertical
    overlap), a warm-up call of warm_steps steps that fills the day-pipelined
    wavefront, then one call of `steps` steady-state steps (forcing and state
    exceed L2).  The warm-up call is launches 0-50 of k_vertical_ahead|k_pipeline
    (one vertical-ahead launch, 50 wavefront launches); the second call starts
    with its vertical-ahead launch (51) and wavefront launches that carry the
    next chunk's vertical balance (52, 53, ...).  One kernel per capture:
      ncu --set full --clock-control none -k regex:k_pipeline -s 50 -c 2 -o prof python bench.py --profile
      ncu --set full --clock-control none -k regex:k_vertical_ahead -s 1 -c 1 -o prof python bench.py --profile
    With outputs (--profile-outputs) the run fills every monthly grid of routing
    and the vertical balance (the same launches, their output variants)."""
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_global()
    nd = (warm_steps + steps) * WAVEFRONT_DAYS
    P, T, S = sy.forcing(region, nd, seed=2, doy0=1)
    m = Model(region, max_days=nd, days_per_step=WAVEFRONT_DAYS)
    if outputs:
        m.monthly_outputs(nd // 28 + 1, doy_day0=1)
        m.monthly_outputs_vertical(True)
        m.monthly_outputs_routing(True)
    m.upload_forcing(0, P, T, S)
    m.run_steps(1, 0, nd, 0, warm_steps)
    m.synchronize()
    t0 = time.perf_counter()
    m.run_steps(1, 0, nd, warm_steps, warm_steps + steps)
    m.synchronize()
    dt = time.perf_counter() - t0
    m.run_steps(1, 0, nd, warm_steps + steps, m.num_steps(nd))
    m.synchronize()
    print(json.dumps({"profile_case": "global grid, steady-state wavefront" + (", monthly grids" if outputs else ""),
                      "ncell": region.ncell, "steps": steps,
                      "days_per_step": WAVEFRONT_DAYS, "seconds": dt,
                      "cell_days_per_s": region.ncell * steps * WAVEFRONT_DAYS / dt, "chunk_steps": m.chunk_steps(),
                      "vertical_overlap_warps": m.vertical_overlap(), "vinline_fraction": m.vinline_fraction()}))


def run_profile_wuse(steps: int = 24, warm_steps: int = 200):
    """The ncu case of the water-use wavefront, as the bench runs it: the global
    grid with water use (three years of synthetic tables), FP64,
    WAVEFRONT_DAYS days per wavefront step, default chunks of 4 steps, vertical
    overlap; launches as in run_profile_case:
      ncu --set full --clock-control none -k regex:k_pipeline -s 50 -c 2 -o prof python bench.py --profile-wuse"""
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_global()
    nd = (warm_steps + steps) * WAVEFRONT_DAYS
    P, T, S = sy.forcing(region, nd, seed=2, doy0=1)
    nus, nug, wdr, cons, frgi = sy.water_use_inputs(region, (nd + 364) // 365)
    m = Model(region, max_days=nd, water_use=True, days_per_step=WAVEFRONT_DAYS)
    m.upload_forcing(0, P, T, S)
    m.set_water_use_inputs(frgi)
    m.upload_water_use_run(0, 1, nd, (nus, nug, wdr, cons))
    m.run_steps(1, 0, nd, 0, warm_steps)
    m.synchronize()
    t0 = time.perf_counter()
    m.run_steps(1, 0, nd, warm_steps, warm_steps + steps)
    m.synchronize()
    dt = time.perf_counter() - t0
    print(json.dumps({"profile_case": "water use, steady-state wavefront", "ncell": region.ncell,
                      "steps": steps, "days_per_step": WAVEFRONT_DAYS, "seconds": dt,
                      "cell_days_per_s": region.ncell * steps * WAVEFRONT_DAYS / dt, "chunk_steps": m.chunk_steps(),
                      "vertical_overlap_warps": m.vertical_overlap()}))


def run_fine():
    """--fine: fine_workload over WG_FINE_YEARS (default 5) simulated years."""
    import torch
    torch.cuda.set_device(0)
    print(json.dumps(fine_workload(int(os.environ.get("WG_FINE_YEARS", "5")))), flush=True)


def fine_workload(years, device=0):
    """Mixed precision at fine resolution: the 5-arc-minute grid (~2.2 M cells),
    FP32 state and fluxes with FP64 confluence and balance sums against the FP64
    run of the same inputs over `years` simulated years; discharge error at every
    outlet and storage error at the end, and the throughput of both precisions
    (one wavefront over the whole run, forcing resident in HBM)."""
    import torch
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    t_all = time.perf_counter()
    region = sy.region_5min()
    t_gen = time.perf_counter() - t_all
    nd = 365 * years
    models = {"fp64": Model(region, max_days=nd, device=device),
              "fp32": Model(region, max_days=nd, precision="fp32", device=device)}
    for y in range(years):
        def up(f, y=y):
            for m in models.values():
                m.upload_forcing(365 * y, f[0], f[1], f[2])
            for m in models.values():
                m.synchronize()
        sy.forcing_year_parallel(region, y, seed=43, consume=up)
    t_setup = time.perf_counter() - t_all
    res = {}
    for name, m in models.items():
        total = m.num_steps(nd)
        m.kernel_timing(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        m.synchronize()
        t0 = time.perf_counter()
        m.run_steps(1, 0, nd, 0, total)
        m.synchronize()
        dt = time.perf_counter() - t0
        kt = m.kernel_times()
        res[name] = {"seconds": dt, "cell_days_per_s": region.ncell * nd / dt, "kernel_ms": kt,
                     "launch_shape": m.launch_shape(), "chunk_steps": m.chunk_steps()}
    q64 = models["fp64"].discharge(0, nd)
    q32 = models["fp32"].discharge(0, nd)
    err_q = outlet_errors(q32, q64)
    # which outlets carry the largest errors: their basins' size and water bodies
    scale = np.maximum(np.abs(q64).max(axis=0), 1e-30)
    daily = np.abs(q32 - q64).max(axis=0) / scale
    mean_e = np.abs(q32.mean(axis=0) - q64.mean(axis=0)) / np.maximum(np.abs(q64.mean(axis=0)), 1e-30)
    from watergap2_gb300.basins import dfs_order
    order, tin, tout = dfs_order(region.downstream)
    st = models["fp64"].stations
    wb = {"reservoirs": region.res_area > 0, "global_lakes": region.lake_area > 0, "local_lakes": region.loc_lake > 0,
          "arid": region.aindex == 1}
    worst = []
    for j in np.argsort(-mean_e)[:5]:
        cells = order[tin[st[j]]:tout[st[j]] + 1]
        worst.append({"basin_cells": int(cells.size), "mean_q": float(q64[:, j].mean()), "mean_err": float(mean_e[j]),
                      "daily_err": float(daily[j]), **{k: int(v[cells].sum()) for k, v in wb.items()}})
    err_q["frac_mean_err_above_1e-5"] = float((mean_e > 1e-5).mean())
    err_q["frac_daily_err_above_1e-5"] = float((daily > 1e-5).mean())
    err_q["worst_outlets"] = worst
    st64, st32 = models["fp64"].get_state(), models["fp32"].get_state()
    err_s = {}
    for k in ("canopy", "snow", "soil", "gw", "river", "loclake", "locwetl", "glolake", "glowetl", "res"):
        a, b = np.asarray(st32[k], np.float64), np.asarray(st64[k], np.float64)
        scale = np.abs(b).max()
        if scale > 0:
            rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-6 * scale)
            err_s[k] = {"max_abs_over_max": float(np.abs(a - b).max() / scale), "rel_q99": float(np.quantile(rel, 0.99))}
    line = {"workload": f"mixed precision, 5-arc-minute grid 2160 x 4320, {region.ncell} cells, "
                        f"{models['fp64'].num_levels} drainage levels, {years} years",
            "metric": "FP32 (FP64 sums) vs FP64: discharge error at every outlet, storage error, cell-days/s",
            "ncell": region.ncell, "outlets": int(q64.shape[1]), "days": nd, "fp64": res["fp64"], "fp32": res["fp32"],
            "fp32_speedup": res["fp32"]["cell_days_per_s"] / res["fp64"]["cell_days_per_s"],
            "discharge_error": err_q, "storage_error_end": err_s, "grid_seconds": t_gen, "setup_seconds": t_setup,
            "data": "synthetic (seeded generators; forcing in parallel chunks, seed 43)"}
    del models
    return line


def run_calibration():
    """--calibration: calibration_workload printed."""
    import torch
    torch.cuda.set_device(0)
    print(json.dumps(calibration_workload()), flush=True)


def calibration_workload(device=0):
    """Calibration workload: 1,000 basins cut from the global drainage tree, gamma
    and CFA calibrated to targets from hidden true parameters, by the reference's
    bisection and by the learned proposer (the plain FP64 model checking every step)."""
    from watergap2_gb300.calibration import run_workload
    out = run_workload(nbasin=1000, lo=20, hi=20000, ndays=730, epochs=40, device=device,
                       log=lambda *a: print(*a, file=sys.stderr, flush=True))
    return {"workload": "learned calibration: 1,000 basins (cells log-uniform 20..20,000, capped at the largest "
                        "basin of the tree), gamma in [0.1, 5], CFA in [0.5, 1.5], 1 % discharge criterion, "
                        "2-year runs (1 spin-up, 1 evaluated)",
            "metric": "calibrations/hour and plain-model calls per basin", **out}


def run_profile_ensemble(members: int = 64, steps: int = 12, warm_steps: int = 200):
    """A short case for ncu of the ensemble kernels: 64 members of the global grid
    (a warp is 32 members of one cell, as with 256), as the bench runs them:
    five days per wavefront step, 128 threads per block and 12-step chunks (the
    autotuner's choice on GB300), a 60-day ring so that the case holds ~2.5 GB
    on the device; a warm-up call of warm_steps steps (17 launch pairs) that
    fills the wavefront, then one call of `steps` steps (one
    k_vertical_ahead<float,1> and one k_pipeline<float,1,1> launch), one kernel per capture:
      ncu --set full --clock-control none -k regex:k_pipeline -s 17 -c 1 -o prof python bench.py --profile-ensemble
      ncu --set full --clock-control none -k regex:k_vertical_ahead -s 17 -c 1 -o prof python bench.py --profile-ensemble"""
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_global()
    nd = (warm_steps + steps) * WAVEFRONT_DAYS
    P, T, S = sy.forcing(region, nd, seed=2, doy0=1)
    pf = np.array([np.exp(np.random.default_rng((7, m)).normal(0.0, 0.3)) for m in range(members)], np.float32)
    m = Model(region, max_days=nd, precision="fp32", members=members, prec_factor=pf, block_threads=128,
              ring_days=60, days_per_step=WAVEFRONT_DAYS)
    m.chunk_steps(steps)
    m.upload_forcing(0, P, T, S)
    m.run_steps(1, 0, nd, 0, warm_steps)
    m.synchronize()
    t0 = time.perf_counter()
    m.run_steps(1, 0, nd, warm_steps, warm_steps + steps)
    m.synchronize()
    dt = time.perf_counter() - t0
    print(json.dumps({"profile_case": "ensemble, steady-state wavefront", "members": members, "ncell": region.ncell,
                      "steps": steps, "days_per_step": WAVEFRONT_DAYS, "seconds": dt,
                      "member_cell_days_per_s": members * region.ncell * steps * WAVEFRONT_DAYS / dt}))


def run_profile_wtemp(steps: int = 24, warm_steps: int = 200):
    """A short case for ncu of the water-temperature wavefront, as the bench
    runs it: the global grid with fractional routing and the water temperature,
    FP64, WAVEFRONT_DAYS days per wavefront step, default chunks of 4 steps,
    vertical overlap.  A warm-up call of warm_steps steps fills the wavefront
    (launches 0-50 of k_vertical_ahead|k_pipeline); the second call starts with
    its vertical-ahead launch (51) and wavefront launches that carry the next
    chunk's vertical balance (52, 53, ...):
      ncu --set full --clock-control none -k regex:k_pipeline -s 50 -c 2 -o prof python bench.py --profile-wtemp"""
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_global().with_options(frac_routing=1)
    nd = (warm_steps + steps) * WAVEFRONT_DAYS
    P, T, S = sy.forcing(region, nd, seed=2, doy0=1)
    LW, GWT = sy.water_temp_inputs(region, nd, T)
    m = Model(region, max_days=nd, water_temp=True, days_per_step=WAVEFRONT_DAYS)
    m.upload_forcing(0, P, T, S)
    m.upload_longwave(0, LW)
    m.set_water_temp_inputs(GWT)
    m.run_steps(1, 0, nd, 0, warm_steps)
    m.synchronize()
    t0 = time.perf_counter()
    m.run_steps(1, 0, nd, warm_steps, warm_steps + steps)
    m.synchronize()
    dt = time.perf_counter() - t0
    print(json.dumps({"profile_case": "water temperature, steady-state wavefront", "ncell": region.ncell,
                      "steps": steps, "days_per_step": WAVEFRONT_DAYS, "seconds": dt,
                      "cell_days_per_s": region.ncell * steps * WAVEFRONT_DAYS / dt, "chunk_steps": m.chunk_steps(),
                      "vertical_overlap_warps": m.vertical_overlap()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile", action="store_true", help="run the short ncu case and exit")
    ap.add_argument("--profile-ensemble", action="store_true", help="run the short ensemble ncu case and exit")
    ap.add_argument("--profile-wtemp", action="store_true", help="run the short water-temperature ncu case and exit")
    ap.add_argument("--profile-wuse", action="store_true", help="run the short water-use ncu case and exit")
    ap.add_argument("--profile-outputs", action="store_true",
                    help="run the short ncu case with the monthly output grids and exit")
    ap.add_argument("--fine", action="store_true",
                    help="the 5-arc-minute mixed-precision run: FP32 vs FP64 errors at every outlet")
    ap.add_argument("--calibration", action="store_true",
                    help="the learned-calibration workload (1,000 basins): bisection vs network proposals")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.profile or args.profile_outputs:
        run_profile_case(outputs=args.profile_outputs)
        return
    if args.calibration:
        run_calibration()
        return
    if args.profile_wtemp:
        run_profile_wtemp()
        return
    if args.profile_wuse:
        run_profile_wuse()
        return
    if args.profile_ensemble:
        run_profile_ensemble()
        return
    if args.fine:
        run_fine()
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    # forcing first (spawned workers), then CUDA
    args.forcing = make_forcing(args.warmup + args.steps)
    run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
