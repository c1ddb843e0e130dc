"""Run the reference's own code (oracle/_ref/wg_ref_harness) on a synthetic region.

TEST INFRASTRUCTURE ONLY, and usable only where the reference sources exist
(the build container): the harness is compiled from them by ``make ref``.  It
writes the region as the input files the reference reads (big-endian UNF grids,
LAI_22.DAT, LCT_22.DAT, a parameter JSON), runs the harness over ``ndays`` and
returns the dumped state.  The reference always has 67,420 grid cells (def.h:10);
the region occupies the first ``ncell`` of them and the rest are marked
non-continental.
"""
from __future__ import annotations

import json
import os
import subprocess
import tempfile

import numpy as np

from watergap2_gb300.region import NPARAM, PARAM_JSON_KEYS

NG = 67420
REF_BANDS = 100
_HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(_HERE, "_ref", "wg_ref_harness")
SNAP_FIELDS = ["canopy", "soil", "snow", "lai_days", "lai_status", "lai_precsum", "gw", "river", "loclake",
               "locwetl", "glolake", "glowetl", "res", "rf_loclake", "rf_locwetl", "rf_glolake", "rf_glowetl",
               "rf_res", "k_release", "laf", "laf_prev", "rs", "gwr"]


def available() -> bool:
    return os.path.exists(HARNESS)


def build(src: str | None = None) -> bool:
    """Compile the harness from the reference's sources in `src` (default: the
    WG_REFERENCE_SOURCE environment variable); False where there are none."""
    src = src or os.environ.get("WG_REFERENCE_SOURCE")
    if not src or not os.path.isdir(src):
        return False
    subprocess.run(["make", "-s", "-C", _HERE, "-j8", "ref", f"REF={src}"], check=True)
    with open(os.path.join(_HERE, "_ref", "source_dir.txt"), "w") as f:
        f.write(os.path.abspath(src))
    return True


def source_dir() -> str | None:
    """The reference source directory the harness was last built from (None if
    it was not built here or the sources are gone)."""
    path = os.path.join(_HERE, "_ref", "source_dir.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        src = f.read().strip()
    return src if os.path.isdir(src) else None


def _unf(path, arr, dt):
    np.asarray(arr).astype(dt).astype(np.dtype(dt).newbyteorder(">")).tofile(path)


def _full(values, dtype, fill=0):
    out = np.full(NG, fill, dtype)
    out[: values.shape[0]] = values
    return out


WU_FIELDS = ["wu_remaining", "wu_unsat_irrig", "wu_unsat_other", "wu_reduced_return", "wu_irrig_withdrawal",
             "wu_irrig_consumptive", "wu_total_unsat", "wu_unsat_prev", "wu_unsat_irrig_prev", "wu_unsat_other_prev",
             "wu_reduced_return_prev", "wu_actual"]
WT_FIELDS = ["wt_river", "wt_loclake", "wt_locwetl", "wt_glolake", "wt_res", "wt_glowetl",
             "ice_river", "ice_loclake", "ice_locwetl", "ice_glolake", "ice_res", "ice_glowetl", "river_avail"]


# the monthly output grids the harness dumps with outputs=1 or 2 (in its order):
# the vertical balance's (daily.cpp:1281-1386; storages at the month's end; total PET
# daily.cpp:1303) and routing's (routing.cpp:3964-4040, storages at the month's end
# 4725-4737)
MONTHLY_VERTICAL = ["prec", "temp", "ext_rad", "short_up_rad", "short_down_rad", "net_short_rad", "net_long_rad",
                    "net_rad", "open_water_pet", "pet", "aet", "land_aet", "land_aet_uncorr", "lai", "albedo",
                    "interception", "canopy_wc", "max_canopy_wc", "snowfall", "rainfall", "snowmelt", "snow_evap",
                    "swe", "snow_cover", "soil_wc", "runoff", "urban_runoff", "surface_runoff", "gw_recharge",
                    "canopy_storage", "snow_storage", "soil_storage", "total_pet"]
# the daily 365 grids of the vertical balance the harness dumps with outputs=2
DAILY_VERTICAL = ["prec", "temp", "pet", "total_pet", "lai", "kc", "albedo", "interception", "canopy_wc",
                  "max_canopy_wc", "snowfall", "snowmelt", "swe", "snow_cover", "soil_wc", "surface_runoff",
                  "gw_recharge", "ext_rad", "short_down_rad", "short_up_rad", "net_short_rad", "net_long_rad",
                  "net_rad", "canopy_storage", "snow_storage", "soil_storage"]
MONTHLY_ROUTING = ["river_avail", "min_river_avail", "max_river_avail", "cell_runoff", "velocity", "loclake_storage",
                   "locwetl_storage", "glolake_storage", "glowetl_storage", "res_storage", "river_storage",
                   "gw_storage", "open_water_evap", "cell_surface_runoff", "gw_runoff", "land_area_frac",
                   "loc_wetl_extent", "glo_wetl_extent", "res_inflow", "res_outflow", "consistent_precip",
                   "surf_storage", "actual_use", "nug", "cell_aet", "cell_aet_wca"]
# with the water temperature, the monthly mean temperatures of the river and the
# five kinds of water body (routing.cpp:4375-4458; -9999 without a computed day)
MONTHLY_WTEMP = ["wt_river", "wt_loclake", "wt_locwetl", "wt_glolake", "wt_res", "wt_glowetl"]
# routing's daily 365 grids the harness dumps with outputs=2
DAILY_ROUTING = ["river_avail", "velocity", "cell_runoff", "cell_runoff_mm", "cell_surface_runoff", "gw_runoff",
                 "land_area_frac", "consistent_precip", "cell_aet"]


def write_case(region, d: str, P, T, S, doy0: int, stations, snapshots, year0: int = 2000, wtemp=None, wuse=None,
               delayed=False, glwd_unit=None, outputs=0):
    n = region.ncell
    if n > NG:
        raise ValueError("region larger than the reference grid")
    reg = region if region.nband == REF_BANDS else region.with_bands(REF_BANDS)
    resopt = int(np.any(region.res_area > 0))
    os.makedirs(os.path.join(d, "G_RES"), exist_ok=True)
    rows = region.row.astype(np.int16)
    cols = region.col.astype(np.int16)
    # geometry (geo.init, source/geo.cpp:7-81)
    area_rows = np.zeros(360, np.float32)
    area_rows[rows - 1] = region.area_km2.astype(np.float32)
    _unf(f"{d}/GAREA.UNF0", area_rows, np.float32)
    _unf(f"{d}/GR.UNF2", _full(rows, np.int16, 1), np.int16)
    _unf(f"{d}/GC.UNF2", _full(cols, np.int16, 1), np.int16)
    _unf(f"{d}/GCRC.UNF4", np.zeros(360 * 720, np.int32), np.int32)
    _unf(f"{d}/GCONTFREQ.UNF0", _full(region.contfreq, np.float32), np.float32)
    f32 = lambda name: _full(region.arrays[name], np.float32)
    _unf(f"{d}/G_LOCLAK.UNF0", f32("loc_lake"), np.float32)
    _unf(f"{d}/G_GLOLAK.UNF0", f32("glo_lake"), np.float32)
    _unf(f"{d}/G_LOCWET.UNF0", f32("loc_wetl"), np.float32)
    _unf(f"{d}/G_GLOWET.UNF0", f32("glo_wetl"), np.float32)
    _unf(f"{d}/G_LOCRES.UNF0", np.zeros(NG, np.float32), np.float32)
    _unf(f"{d}/G_RES/G_RES_FRAC.UNF0", f32("glo_res"), np.float32)
    _unf(f"{d}/G_RES/G_RES_2000.UNF0", f32("glo_res"), np.float32)
    _unf(f"{d}/G_LAKAREA.UNF0", f32("lake_area"), np.float32)
    _unf(f"{d}/G_RESAREA.UNF0", f32("res_area"), np.float32)
    _unf(f"{d}/G_REGLAKE.UNF0", np.zeros(NG, np.float32), np.float32)
    _unf(f"{d}/G_REG_LAKE.UNF1", np.zeros(NG, np.int8), np.int8)
    _unf(f"{d}/G_OUTFLOW_CELL_ASSIGNMENT.UNF4", np.zeros(NG, np.int32), np.int32)
    down = _full(region.downstream.astype(np.int32) + 1, np.int32)     # 1-based, 0 = outlet
    down[down < 0] = 0
    _unf(f"{d}/G_OUTFLC.UNF4", down, np.int32)
    _unf(f"{d}/G_RES_TYPE.UNF1", _full(region.res_type, np.int8, 2), np.int8)
    _unf(f"{d}/G_START_YEAR.UNF4", np.full(NG, 1900, np.int32), np.int32)
    _unf(f"{d}/G_START_MONTH.UNF1", _full(region.start_month, np.int8, 1), np.int8)
    _unf(f"{d}/G_MEAN_OUTFLOW.UNF0", _full(region.extras["mean_outflow_km3_month"], np.float32), np.float32)
    _unf(f"{d}/G_STORAGE_CAPACITY.UNF0", f32("stor_cap"), np.float32)
    _unf(f"{d}/G_NUs_1971_2000.UNF0", np.zeros(NG, np.float32), np.float32)
    _unf(f"{d}/G_ALLOC_COEFF.5.UNF0", np.zeros(NG * 5, np.float32), np.float32)
    _unf(f"{d}/G_RIVER_LENGTH.UNF0", _full(region.extras["river_length_file"], np.float32, 50.0), np.float32)
    _unf(f"{d}/G_RIVERSLOPE.UNF0", _full(region.river_slope, np.float32, 1e-3), np.float32)
    _unf(f"{d}/G_ROUGHNESS.UNF0", _full(region.roughness, np.float32, 0.03), np.float32)
    _unf(f"{d}/G_BANKFULL.UNF0", _full(region.bankfull, np.float32, 1.0), np.float32)
    # routing order: G_ROUT_ORDER[cell] = 1-based position; padding cells come last
    pos = np.empty(NG, np.int32)
    pos[region.rout_order] = np.arange(n, dtype=np.int32) + 1
    pos[n:] = np.arange(n, NG, dtype=np.int32) + 1
    _unf(f"{d}/G_ROUT_ORDER.UNF4", pos, np.int32)
    ldd = _full(region.ldd, np.int8, 5)
    _unf(f"{d}/G_LDD_2.UNF1", ldd, np.int8)
    # land-cover tables (LAI_22.DAT: lai.cpp:110-149, LCT_22.DAT: daily.cpp:1925-1959)
    tb = region.lct_tables
    with open(f"{d}/LAI_22.DAT", "w") as f:
        f.write("# synthetic LAI table\n")
        for i in range(18):
            f.write(f"{i + 1} {float(tb['lai'][i])!r} {float(tb['fdp'][i])!r} {float(tb['rfep'][i])!r} "
                    f"{int(tb['initial_days'][i])} {float(tb['kc_min'][i])!r} {float(tb['kc_max'][i])!r}\n")
    with open(f"{d}/LCT_22.DAT", "w") as f:
        f.write("# synthetic land-cover table\n")
        for i in range(18):
            f.write(f"{i + 1} {float(tb['rooting'][i])!r} {float(tb['albedo'][i])!r} "
                    f"{float(tb['albedo_snow'][i])!r} {float(tb['ddf'][i])!r} {float(tb['emissivity'][i])!r}\n")
    par = region.arrays["param"].reshape(NPARAM, n)
    obj = {}
    for k, key in enumerate(PARAM_JSON_KEYS):
        full = np.ones(NG)
        full[:n] = par[k]
        obj[key] = [float(x) for x in full]
    # multipliers of the net abstractions (routing.cpp:910-916), which getValue
    # reads as 0 when absent
    obj["net_abstraction_surfacewater_mult"] = [1.0] * NG
    obj["net_abstraction_groundwater_mult"] = [1.0] * NG
    with open(f"{d}/params.json", "w") as f:
        json.dump(obj, f)
    with open(f"{d}/config.txt", "w") as f:
        f.write(f"routing {d}/ROUTING.DAT\nend_of_head\n")
    # raw arrays the harness sets directly
    region.lct.astype(np.uint8).tofile(f"{d}/c_lct.bin")
    region.built_up.astype(np.float32).tofile(f"{d}/c_built_up.bin")
    region.smax.astype(np.float32).tofile(f"{d}/c_smax.bin")
    region.lai_max.astype(np.float32).tofile(f"{d}/c_lai_max.bin")
    region.gw_factor.astype(np.float32).tofile(f"{d}/c_gw_factor.bin")
    region.rg_max.astype(np.int16).tofile(f"{d}/c_rg_max.bin")
    region.texture.astype(np.int8).tofile(f"{d}/c_texture.bin")
    region.aindex.astype(np.int16).tofile(f"{d}/c_aindex.bin")
    reg.elev.astype(np.int16).tofile(f"{d}/c_elev.bin")
    np.asarray(stations, np.int32).tofile(f"{d}/c_stations.bin")
    np.ascontiguousarray(P, np.float32).tofile(f"{d}/f_prec.bin")
    np.ascontiguousarray(T, np.float32).tofile(f"{d}/f_temp.bin")
    np.ascontiguousarray(S, np.float32).tofile(f"{d}/f_swrad.bin")
    if outputs:   # read by dailyWaterBalanceClass::init with grid_store 2 (daily.cpp:1558)
        _unf(f"{d}/G_ALBEDO_CYCLE.12.UNF0", np.zeros(NG * 12, np.float32), np.float32)
    if wtemp is not None:   # (longwave [ndays, ncell], groundwater temperature [ncell])
        from watergap2_gb300.region import inflow_cells
        lw, gwt = wtemp
        np.ascontiguousarray(lw, np.float32).tofile(f"{d}/f_lwrad.bin")
        np.ascontiguousarray(gwt, np.float32).tofile(f"{d}/c_gwtemp.bin")
        ic = np.zeros((NG, 9), np.int32)
        ic[:n] = inflow_cells(region) + 1           # 1-based, 0 = none
        _unf(f"{d}/G_INFLC.9.UNF4", ic.ravel(), np.int32)
    if wuse is not None:
        # (nus, nug, irrigation withdrawal, irrigation consumptive use: [years, 12, ncell] m3 per month,
        #  fraction of irrigation return flow into groundwater [ncell]); the yearly files dailyNUInit
        #  reads (routing.cpp:892-907), cell-major [cell][month]
        nus, nug, wdr, cons, frgi = wuse
        _unf(f"{d}/G_FRACTRETURNGW_IRRIG.UNF0", _full(np.asarray(frgi), np.float32), np.float32)
        units = np.zeros(NG, np.int32) if glwd_unit is None else _full(np.asarray(glwd_unit), np.int32)
        _unf(f"{d}/GLWDunits.UNF4", units, np.int32)
        for k in range(np.asarray(nus).shape[0]):
            for name, arr in (("G_NETUSE_SW_m3", nus), ("G_NETUSE_GW_m3", nug),
                              ("G_IRRIG_WITHDRAWAL_USE_SW_m3", wdr), ("G_IRRIG_CONS_USE_SW_m3", cons)):
                full = np.zeros((NG, 12), np.float32)
                full[:n] = np.asarray(arr[k], np.float32).T
                _unf(f"{d}/{name}_{year0 + k}.12.UNF0", full.ravel(), np.float32)
    with open(f"{d}/meta.txt", "w") as f:
        f.write(f"{n} {P.shape[0]} {doy0} {year0} {resopt} {region.river_velo_opt} {len(stations)} {len(snapshots)} "
                f"{0 if wtemp is None else 1} {int(getattr(region, 'frac_routing', 0))} "
                f"{0 if wuse is None else (2 if delayed else 1) + (0 if glwd_unit is None else 2)} "
                f"{int(getattr(region, 'statcorr_opt', 0))} {int(outputs)}\n")
    with open(f"{d}/snapshots.txt", "w") as f:
        f.write(" ".join(str(int(s)) for s in snapshots) + "\n")


def run(region, P, T, S, doy0=1, stations=None, snapshots=None, workdir=None, wtemp=None, wuse=None, delayed=False,
        threads=1, glwd_unit=None, outputs=0):
    """Run the reference harness; returns dict(lai_a, lai_b, bottom_width, snapshots=[{field: array}],
    discharge=[ndays, nstation], stations=..., timing=dict(threads, vertical_s, routing_s)): the vertical
    pass on `threads` OpenMP threads, routing serial, as integrate_wghm_ runs them."""
    if not available():
        raise RuntimeError("reference harness not built (make -C oracle ref)")
    ndays = P.shape[0]
    n = region.ncell
    if stations is None:
        outl = np.nonzero((region.downstream < 0) & (region.ldd >= 0))[0]
        stations = outl[:40]
    stations = np.asarray(stations, np.int32)
    snapshots = list(snapshots or [ndays])
    tmp = workdir or tempfile.mkdtemp(prefix="wg_ref_")
    write_case(region, tmp, P, T, S, doy0, stations, snapshots, wtemp=wtemp, wuse=wuse, delayed=delayed,
               glwd_unit=glwd_unit, outputs=outputs)
    out = os.path.join(tmp, "out.bin")
    env = dict(os.environ, WG_REF_THREADS=str(int(threads)))
    subprocess.run([HARNESS, tmp, out], check=True, stdout=subprocess.DEVNULL, env=env)
    raw = np.fromfile(out, np.float64)
    o = 0
    res = {"lai_a": raw[o:o + 18].copy(), "lai_b": raw[o + 18:o + 36].copy()}
    o += 36
    res["bottom_width"] = raw[o:o + n].copy(); o += n
    o += n   # land fraction before the first annualInit (unused)
    snaps = []
    for _ in snapshots:
        snap = {}
        for f in SNAP_FIELDS:
            snap[f] = raw[o:o + n].copy(); o += n
        bands = raw[o:o + REF_BANDS * n].reshape(REF_BANDS, n).T.copy(); o += REF_BANDS * n
        snap["snow_band"] = bands
        if wtemp is not None:
            for f in WT_FIELDS:
                snap[f] = raw[o:o + n].copy(); o += n
        if wuse is not None:
            for f in WU_FIELDS + (["wu_unsat_riparian"] if glwd_unit is not None else []):
                snap[f] = raw[o:o + n].copy(); o += n
        snaps.append(snap)
    res["snapshots"] = snaps
    res["discharge"] = raw[o:o + ndays * len(stations)].reshape(ndays, len(stations)).copy()
    o += ndays * len(stations)
    if wtemp is not None:
        res["river_temp"] = raw[o:o + ndays * len(stations)].reshape(ndays, len(stations)).copy()
        o += ndays * len(stations)
    if outputs:   # the year's monthly grids [12][ncell] per field
        res["monthly"] = {}
        for f in MONTHLY_VERTICAL + MONTHLY_ROUTING + (MONTHLY_WTEMP if wtemp is not None else []):
            res["monthly"][f] = raw[o:o + 12 * n].reshape(12, n).copy()
            o += 12 * n
    if outputs == 2:   # the year's daily grids [365][ncell] per field
        res["daily"] = {}
        for f in DAILY_VERTICAL + ["r_" + k for k in DAILY_ROUTING]:
            res["daily"][f] = raw[o:o + 365 * n].reshape(365, n).copy()
            o += 365 * n
    assert o == raw.size, (o, raw.size)
    res["stations"] = stations
    with open(os.path.join(tmp, "timing.txt")) as f:
        th, tv, tr = f.read().split()[:3]
    res["timing"] = {"threads": int(th), "vertical_s": float(tv), "routing_s": float(tr)}
    return res
