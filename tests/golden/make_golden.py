"""Regenerate the golden fixtures from the reference's own code.

Runs only where the reference sources are present (the build container): it
builds oracle/_ref/wg_ref_harness from them (oracle/Makefile, target "ref"),
runs each case below through the reference's calcNewDay/routing, and stores
the inputs together with the reference's outputs, so that the tests can check
the C restatement -- and through it the GPU library -- on any machine.

    python tests/golden/make_golden.py [case ...]

The water-temperature case (WT_CASES) adds longwave radiation, groundwater
temperature and the reference's inflow-direction table to the inputs; the
water-use case (WU_CASES) adds three years of monthly net abstractions.
"""
import dataclasses
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

sys.path.insert(0, os.path.join(ROOT, "tests"))
from oracle import ref_case  # noqa: E402
from watergap2_gb300 import synthetic as sy  # noqa: E402
from watergap2_gb300.region import save_npz  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference's sources (WG_REFERENCE_SOURCE, else the build container's mount)
REF_SOURCE = os.environ.get("WG_REFERENCE_SOURCE") or "/root/reference/source"

# name -> (region factory, days, first day of year, snapshot days)
CASES = {
    "region16_365d": (lambda: sy.region_64x64(seed=1, size=16), 365, 1, [1, 180, 365]),
    "region64_30d": (lambda: sy.region_64x64(seed=1), 30, 1, [30]),
    "swb_velo1_200d": (lambda: sy.region_small_swb(seed=21), 200, 20, [100, 200]),
    "swb_velo2_120d": (lambda: sy.region_small_swb(seed=5, ny=16, nx=32, river_velo_opt=2), 120, 300, [120]),
    # fractional routing (options.fractionalRoutingOpt = 1) on a block of the 0.5-degree grid
    "swb_frac_150d": (lambda: sy.region_small_swb(seed=33, block_at=(150, 420)).with_options(frac_routing=1),
                      150, 60, [75, 150]),
    # station correction (options.statcorrOpt = 1): outflow x P_CFS (routing.cpp:3929-3931)
    "swb_statcorr_120d": (lambda: statcorr_region(seed=22), 120, 150, [60, 120]),
    # cells without continental area (G_contcell = 0, geo.cpp:50-60): no vertical balance
    "swb_nocont_150d": (lambda: nocont_region(seed=23), 150, 100, [75, 150]),
}


def statcorr_region(seed=22):
    """A region with every water-body type whose cells carry station correction
    factors P_CFS: 1 in most cells (as the reference sets them outside its
    calibration stations), U(0.6, 1.4) in every fifth cell."""
    region = sy.region_small_swb(seed=seed, block_at=(120, 200))
    rng = np.random.default_rng(seed + 100)
    f = np.ones(region.ncell)
    f[::5] = rng.uniform(0.6, 1.4, f[::5].size)
    return region.with_param("P_CFS", f).with_options(statcorr_opt=1)


def main(names=None):
    if not ref_case.available():
        if not ref_case.build(REF_SOURCE):
            raise SystemExit("reference sources not found; cannot regenerate fixtures")
    for name, (make, nd, doy0, snaps) in CASES.items():
        if names and name not in names:
            continue
        region = make()
        P, T, S = sy.forcing(region, nd, doy0=doy0)
        outl = np.nonzero((region.downstream < 0) & (region.ldd >= 0))[0]
        stations = outl[:24]
        res = ref_case.run(region, P, T, S, doy0=doy0, stations=stations, snapshots=snaps)
        extra = dict(P=P, T=T, S=S, doy0=np.array(doy0), stations=res["stations"], snap_days=np.array(snaps),
                     discharge=res["discharge"])
        _put_snapshots(region, res, extra)
        path = os.path.join(HERE, f"{name}.npz")
        save_npz(region, path, **extra)
        print(f"{name}: {region.ncell} cells x {nd} days -> {os.path.getsize(path) / 1e6:.2f} MB")


def _put_snapshots(region, res, extra):
    """The reference's state at each snapshot day as s<i>_<field>, one snow band
    of each replicated group."""
    rep = ref_case.REF_BANDS // region.nband
    for i, snap in enumerate(res["snapshots"]):
        bands = snap.pop("snow_band")
        # replicated bands must agree with each other; keep one per band
        b = bands.reshape(region.ncell, region.nband, rep)
        assert np.array_equal(b, np.repeat(b[:, :, :1], rep, axis=2))
        extra[f"s{i}_snow_band"] = b[:, :, 0].copy()
        for k, v in snap.items():
            extra[f"s{i}_{k}"] = v


def nocont_region(seed=23):
    """A region with every water-body type in which five cells have a continental
    share below the reference's limit (1e-6 %), as the Caspian Sea's cells in the
    standard land mask: two global lakes, a local wetland and a cell without water
    bodies at 0 %, and one cell without water bodies at 5e-7 %.  The reference runs
    no vertical balance in them (integrateWGHM.cpp:770-780)."""
    region = sy.region_small_swb(seed=seed, block_at=(90, 260))
    a = region.arrays
    plain = (a["lake_area"] == 0) & (a["res_area"] == 0) & (a["loc_lake"] == 0) & (a["loc_wetl"] == 0) & \
        (a["glo_wetl"] == 0)
    pick = [np.nonzero(a["lake_area"] > 0)[0][:2], np.nonzero((a["loc_wetl"] > 0) & (a["lake_area"] == 0))[0][:1],
            np.nonzero(plain)[0][:2]]
    cf = a["contfreq"].copy()
    cf[np.concatenate(pick[:2] + [pick[2][:1]])] = 0.0
    cf[pick[2][1]] = float(np.float32(5e-7))   # the reference reads the share as float
    arrays = dict(a)
    arrays["contfreq"] = cf
    # the river length scaled by the continental share as geo.init raises it to the
    # lake and reservoir share (routing.cpp:476-482, geo.cpp:25-45)
    share = np.maximum(cf, ((a["loc_lake"] + a["glo_lake"]) + 0.0) + a["glo_res"])
    arrays["river_length"] = region.extras["river_length_file"] * (share / 100.)
    out = dataclasses.replace(region, arrays=arrays)
    for k in ("lct_tables", "extras"):
        if k in region.__dict__:
            out.__dict__[k] = region.__dict__[k]
    return out


def wtemp_region(seed=21):
    """A 24 x 48 block of the 0.5-degree grid with every water-body type; a third
    of its inland sinks carry the reference's no-river marker (river length 55 in
    the input file), so that the water temperature routes their local runoff into
    the cell's water bodies."""
    region = sy.region_small_swb(seed=seed, block_at=(100, 300))
    raw = region.extras["river_length_file"].copy()
    sinks = np.nonzero(region.downstream < 0)[0]
    raw[sinks[::3]] = 55.0
    region.extras["river_length_file"] = raw
    region.arrays["river_length"] = raw * (region.contfreq / 100.)      # routing.cpp:480-482
    # the reference's option parser switches fractional routing on with calc_wtemp
    # (option.cpp:591-593)
    return region.with_options(frac_routing=1)


# water temperature: name -> (region factory, days, first day of year, snapshot days)
WT_CASES = {
    "swb_wtemp_90d": (wtemp_region, 90, 240, [45, 90]),
}


def main_wtemp(names=None):
    if not ref_case.available():
        if not ref_case.build(REF_SOURCE):
            raise SystemExit("reference sources not found; cannot regenerate fixtures")
    for name, (make, nd, doy0, snaps) in WT_CASES.items():
        if names and name not in names:
            continue
        region = make()
        P, T, S = sy.forcing(region, nd, doy0=doy0)
        T = (T - 9.0).astype(np.float32)     # a cold autumn: ice forms, grows and breaks up
        LW, GWT = sy.water_temp_inputs(region, nd, T)
        outl = np.nonzero((region.downstream < 0) & (region.ldd >= 0))[0]
        stations = outl[:24]
        res = ref_case.run(region, P, T, S, doy0=doy0, stations=stations, snapshots=snaps, wtemp=(LW, GWT))
        extra = dict(P=P, T=T, S=S, LW=LW, GWT=GWT, doy0=np.array(doy0), stations=res["stations"],
                     snap_days=np.array(snaps), discharge=res["discharge"], river_temp=res["river_temp"])
        for i, snap in enumerate(res["snapshots"]):
            snap.pop("snow_band")
            for k in ref_case.WT_FIELDS + ["river", "soil", "gw"]:
                extra[f"s{i}_{k}"] = snap[k]
        path = os.path.join(HERE, f"{name}.npz")
        save_npz(region, path, **extra)
        print(f"{name}: {region.ncell} cells x {nd} days -> {os.path.getsize(path) / 1e6:.2f} MB")


# water use (options.subtract_use = 2, satisfied in the cell itself):
# name -> (region factory, days, first day of year, snapshot days, water-use seed[, delayed])
WU_CASES = {
    # two year ends (days 36 and 401): annualWaterUsePostProcessing and annualInit
    "swb_wuse_420d": (lambda: sy.region_small_swb(seed=21, ny=16, nx=32, block_at=(100, 300)), 420, 330,
                      [36, 200, 401, 420], 13),
    # with fractional routing (the groundwater variants of routing.cpp:1986-2146 take NUg too)
    "swb_wuse_frac_200d": (lambda: sy.region_small_swb(seed=34, ny=16, nx=32, block_at=(150, 420))
                           .with_options(frac_routing=1), 200, 200, [166, 200], 17),
    # delayed satisfaction (options.delayedUseSatisfaction = 1): unmet demand adds to the next day's
    "swb_wuse_delayed_420d": (lambda: sy.region_small_swb(seed=21, ny=16, nx=32, block_at=(100, 300)), 420, 330,
                              [36, 200, 401, 420], 13, True),
}


def main_wuse(names=None):
    if not ref_case.available():
        if not ref_case.build(REF_SOURCE):
            raise SystemExit("reference sources not found; cannot regenerate fixtures")
    for name, (make, nd, doy0, snaps, seed, *opt) in WU_CASES.items():
        delayed = bool(opt and opt[0])
        if names and name not in names:
            continue
        region = make()
        P, T, S = sy.forcing(region, nd, doy0=doy0)
        nus, nug, wdr, cons, frgi = sy.water_use_inputs(region, 3, seed=seed)
        # most water-body cells abstract more than their lakes and reservoirs hold over a
        # year: local lakes go below zero, reservoirs down to their 10 % floor
        a = region.arrays
        heavy = np.nonzero((a["loc_lake"] > 0) | (a["res_area"] > 0) | (a["lake_area"] > 0))[0][::3]
        keep = np.ones(region.ncell, bool)
        keep[heavy] = False
        nus = np.where(keep[None, None, :], nus, np.abs(nus) * 20.0 + np.float32(3.0e8)).astype(np.float32)
        outl = np.nonzero((region.downstream < 0) & (region.ldd >= 0))[0]
        stations = outl[:24]
        res = ref_case.run(region, P, T, S, doy0=doy0, stations=stations, snapshots=snaps,
                           wuse=(nus, nug, wdr, cons, frgi), delayed=delayed)
        extra = dict(P=P, T=T, S=S, NUS=nus, NUG=nug, WDR=wdr, CONS=cons, FRGI=frgi, doy0=np.array(doy0),
                     delayed=np.array(int(delayed)),
                     stations=res["stations"], snap_days=np.array(snaps), discharge=res["discharge"])
        for i, snap in enumerate(res["snapshots"]):
            snap.pop("snow_band")
            for k in ref_case.WU_FIELDS + ["gw", "river", "loclake", "locwetl", "glolake", "glowetl", "res",
                                           "rf_loclake", "rf_glolake", "rf_res", "k_release", "laf", "soil"]:
                extra[f"s{i}_{k}"] = snap[k]
        path = os.path.join(HERE, f"{name}.npz")
        save_npz(region, path, **extra)
        print(f"{name}: {region.ncell} cells x {nd} days -> {os.path.getsize(path) / 1e6:.2f} MB")


# water use with the NUs of global lakes' and reservoirs' riparian cells met by
# their outflow cell (aggrNUsGloLakResOpt = 1; GLWD units from synthetic.glwd_units):
# name -> (region factory, days, first day of year, snapshot days, water-use seed, delayed)
GLWD_CASES = {
    "swb_wuse_glwd_420d": (lambda: sy.region_small_swb(seed=21, ny=16, nx=32, block_at=(100, 300)), 420, 330,
                           [36, 200, 401, 420], 13, False),
    "swb_wuse_glwd_delayed_200d": (lambda: sy.region_small_swb(seed=34, ny=16, nx=32, block_at=(150, 420)), 200, 120,
                                   [90, 200], 17, True),
}


def main_wuse_glwd(names=None):
    if not ref_case.available():
        if not ref_case.build(REF_SOURCE):
            raise SystemExit("reference sources not found; cannot regenerate fixtures")
    for name, (make, nd, doy0, snaps, seed, delayed) in GLWD_CASES.items():
        if names and name not in names:
            continue
        region = make()
        unit = sy.glwd_units(region)
        P, T, S = sy.forcing(region, nd, doy0=doy0)
        nus, nug, wdr, cons, frgi = sy.water_use_inputs(region, 3, seed=seed)
        # riparian cells abstract more than their lakes and reservoirs can give
        # (unmet aggregated use goes back to them); a few of them return water
        rip = np.nonzero((unit > 0) & (region.lake_area <= 0) & (region.res_area <= 0))[0]
        big = np.abs(nus[:, :, rip]) * 30.0 + np.float32(5.0e8)
        big[:, :, ::5] *= -0.2
        nus = nus.copy()
        nus[:, :, rip] = big.astype(np.float32)
        outl = np.nonzero((region.downstream < 0) & (region.ldd >= 0))[0]
        stations = outl[:24]
        res = ref_case.run(region, P, T, S, doy0=doy0, stations=stations, snapshots=snaps,
                           wuse=(nus, nug, wdr, cons, frgi), delayed=delayed, glwd_unit=unit)
        extra = dict(P=P, T=T, S=S, NUS=nus, NUG=nug, WDR=wdr, CONS=cons, FRGI=frgi, GLWD=unit,
                     doy0=np.array(doy0), delayed=np.array(int(delayed)),
                     stations=res["stations"], snap_days=np.array(snaps), discharge=res["discharge"])
        for i, snap in enumerate(res["snapshots"]):
            snap.pop("snow_band")
            for k in ref_case.WU_FIELDS + ["wu_unsat_riparian", "gw", "river", "loclake", "locwetl", "glolake",
                                           "glowetl", "res", "rf_loclake", "rf_glolake", "rf_res", "k_release", "laf",
                                           "soil"]:
                extra[f"s{i}_{k}"] = snap[k]
        path = os.path.join(HERE, f"{name}.npz")
        save_npz(region, path, **extra)
        print(f"{name}: {region.ncell} cells x {nd} days -> {os.path.getsize(path) / 1e6:.2f} MB")


def main_outputs(names=None, name="swb_outputs_730d"):
    """The monthly output grids (grid_store = 6: monthly, storages at the month's
    end) of the vertical balance and routing, and the vertical balance's daily 365
    grids, on the water-body region with inland sinks over two calendar years: the
    grids hold the second year (annualInit resets them; total PET's freshwater
    share is then the local lakes' share at the year's start, routing.cpp:1249-1259)."""
    if names and name not in names:
        return
    if not ref_case.available():
        if not ref_case.build(REF_SOURCE):
            raise SystemExit("reference sources not found; cannot regenerate fixtures")
    region = sy.region_small_swb(seed=21, ny=16, nx=32, block_at=(100, 300))
    nd = 730
    P, T, S = sy.forcing(region, nd, doy0=1)
    outl = np.nonzero((region.downstream < 0) & (region.ldd >= 0))[0]
    res = ref_case.run(region, P, T, S, doy0=1, stations=outl[:24], snapshots=[nd], outputs=2)
    extra = dict(P=P, T=T, S=S, doy0=np.array(1), stations=res["stations"], snap_days=np.array([nd]),
                 discharge=res["discharge"])
    _put_snapshots(region, res, extra)
    for k, v in res["monthly"].items():
        extra[f"m_{k}"] = v
    # the daily grids on a sample of days (the first days of January and February,
    # every 13th day, the last day), to keep the fixture small
    days = np.unique(np.r_[0:3, 31:34, np.arange(0, 365, 13), 364])
    extra["daily_days"] = days
    for k, v in res["daily"].items():   # the vertical balance's as d_<field>, routing's as d_r_<field>
        extra[f"d_{k}"] = v[days]
    path = os.path.join(HERE, f"{name}.npz")
    save_npz(region, path, **extra)
    print(f"{name}: {region.ncell} cells x {nd} days -> {os.path.getsize(path) / 1e6:.2f} MB")


def main_outputs_wuse(names=None, name="swb_outputs_wuse_730d", glwd=False):
    """The output grids of main_outputs with water use met in the cell
    (subtract_use = 2): the same region, two calendar years, the water-use inputs
    of swb_wuse_420d; the grids hold the second year, among them the monthly
    actual use and NUg (routing.cpp:3744-3747).  glwd: the riparian cells' NUs
    met by their global lake's or reservoir's outflow cell (aggrNUsGloLakResOpt
    = 1, the units of synthetic.glwd_units)."""
    if names and name not in names:
        return
    if not ref_case.available():
        if not ref_case.build(REF_SOURCE):
            raise SystemExit("reference sources not found; cannot regenerate fixtures")
    region = sy.region_small_swb(seed=21, ny=16, nx=32, block_at=(100, 300))
    nd = 730
    P, T, S = sy.forcing(region, nd, doy0=1)
    nus, nug, wdr, cons, frgi = sy.water_use_inputs(region, 3, seed=13)
    outl = np.nonzero((region.downstream < 0) & (region.ldd >= 0))[0]
    unit = sy.glwd_units(region) if glwd else None
    res = ref_case.run(region, P, T, S, doy0=1, stations=outl[:24], snapshots=[nd], outputs=2,
                       wuse=(nus, nug, wdr, cons, frgi), glwd_unit=unit)
    extra = dict(P=P, T=T, S=S, NUS=nus, NUG=nug, WDR=wdr, CONS=cons, FRGI=frgi, doy0=np.array(1),
                 delayed=np.array(0), stations=res["stations"], snap_days=np.array([nd]),
                 discharge=res["discharge"])
    if glwd:
        extra["GLWD"] = unit
    for k, v in res["monthly"].items():
        extra[f"m_{k}"] = v
    days = np.unique(np.r_[0:3, 31:34, np.arange(0, 365, 13), 364])
    extra["daily_days"] = days
    for k, v in res["daily"].items():
        extra[f"d_{k}"] = v[days]
    path = os.path.join(HERE, f"{name}.npz")
    save_npz(region, path, **extra)
    print(f"{name}: {region.ncell} cells x {nd} days -> {os.path.getsize(path) / 1e6:.2f} MB")


def main_outputs_wtemp(names=None, name="swb_outputs_wtemp_365d"):
    """The monthly output grids with the water temperature (calc_wtemp = 1, and so
    fractional routing), among them the monthly mean temperatures of the river and
    every water body, over one calendar year on the water-temperature region."""
    if names and name not in names:
        return
    if not ref_case.available():
        if not ref_case.build(REF_SOURCE):
            raise SystemExit("reference sources not found; cannot regenerate fixtures")
    region = wtemp_region(seed=21)
    nd = 365
    P, T, S = sy.forcing(region, nd, doy0=1)
    T = (T - 9.0).astype(np.float32)     # cold winters: ice forms, grows and breaks up
    LW, GWT = sy.water_temp_inputs(region, nd, T)
    outl = np.nonzero((region.downstream < 0) & (region.ldd >= 0))[0]
    res = ref_case.run(region, P, T, S, doy0=1, stations=outl[:24], snapshots=[nd], wtemp=(LW, GWT), outputs=1)
    extra = dict(P=P, T=T, S=S, LW=LW, GWT=GWT, doy0=np.array(1), stations=res["stations"],
                 snap_days=np.array([nd]), discharge=res["discharge"], river_temp=res["river_temp"])
    for k, v in res["monthly"].items():
        extra[f"m_{k}"] = v
    path = os.path.join(HERE, f"{name}.npz")
    save_npz(region, path, **extra)
    print(f"{name}: {region.ncell} cells x {nd} days -> {os.path.getsize(path) / 1e6:.2f} MB")


def main_wtemp_wuse(names=None, name="swb_wtemp_wuse_120d"):
    """Water use together with the water temperature (calc_wtemp = 1, subtract_use
    = 2): the water-temperature region and a cold season across a year end."""
    if names and name not in names:
        return
    if not ref_case.available():
        if not ref_case.build(REF_SOURCE):
            raise SystemExit("reference sources not found; cannot regenerate fixtures")
    region = wtemp_region(seed=21)
    nd, doy0, snaps = 120, 300, [66, 120]
    P, T, S = sy.forcing(region, nd, doy0=doy0)
    T = (T - 9.0).astype(np.float32)
    LW, GWT = sy.water_temp_inputs(region, nd, T)
    nus, nug, wdr, cons, frgi = sy.water_use_inputs(region, 2, seed=19)
    a = region.arrays
    heavy = np.nonzero((a["loc_lake"] > 0) | (a["res_area"] > 0) | (a["lake_area"] > 0))[0][::3]
    keep = np.ones(region.ncell, bool)
    keep[heavy] = False
    nus = np.where(keep[None, None, :], nus, np.abs(nus) * 20.0 + np.float32(3.0e8)).astype(np.float32)
    outl = np.nonzero((region.downstream < 0) & (region.ldd >= 0))[0]
    stations = outl[:24]
    res = ref_case.run(region, P, T, S, doy0=doy0, stations=stations, snapshots=snaps, wtemp=(LW, GWT),
                       wuse=(nus, nug, wdr, cons, frgi))
    extra = dict(P=P, T=T, S=S, LW=LW, GWT=GWT, NUS=nus, NUG=nug, WDR=wdr, CONS=cons, FRGI=frgi,
                 doy0=np.array(doy0), stations=res["stations"], snap_days=np.array(snaps),
                 discharge=res["discharge"], river_temp=res["river_temp"])
    for i, snap in enumerate(res["snapshots"]):
        snap.pop("snow_band")
        for k in ref_case.WT_FIELDS + ref_case.WU_FIELDS + ["river", "soil", "gw", "loclake", "glolake", "res"]:
            extra[f"s{i}_{k}"] = snap[k]
    path = os.path.join(HERE, f"{name}.npz")
    save_npz(region, path, **extra)
    print(f"{name}: {region.ncell} cells x {nd} days -> {os.path.getsize(path) / 1e6:.2f} MB")


# Workloads whose inputs are too large to store: the fixture keeps the seeds, a
# digest of the regenerated inputs, and the reference's outputs -- the daily
# discharge of a set of stations, every state field of a sample of cells, and
# the exact sum over all cells of every state field at each snapshot.
#   name -> (region factory, days, first day of year, forcing seed, snapshot days,
#            cells sampled at the last snapshot: every k-th cell plus every cell
#            with a water body (None: all cells), station choice)
REGEN_CASES = {
    # the 64 x 64 all-land region over a whole year (one outlet)
    "config1_region64_365d": ("region_64x64", 365, 1, 2, [182, 365], None, "region64"),
    # the global 0.5-degree grid, 67,420 cells, water bodies on, 120 days from 1 January
    "config2_global_120d": ("region_global", 120, 1, 2, [60, 120], 16, "global"),
}
REGEN_KEYS = ["canopy", "soil", "snow", "lai_days", "lai_status", "lai_precsum", "gw", "river", "loclake",
              "locwetl", "glolake", "glowetl", "res", "rf_loclake", "rf_locwetl", "rf_glolake", "rf_glowetl",
              "rf_res", "laf", "laf_prev"]


def regen_stations(region, kind, seed=5):
    """Stations of a regenerated case: for the 64 x 64 region its outlet and every
    64th cell of the routing order; on the global grid the 384 outlets with the
    largest basins, 128 other outlets and 256 interior cells (seeded)."""
    outl = np.nonzero((region.downstream < 0) & (region.ldd >= 0))[0]
    if kind == "region64":
        return np.unique(np.concatenate([outl, region.rout_order[::64]])).astype(np.int32)
    from watergap2_gb300.basins import dfs_order
    order, tin, tout = dfs_order(region.downstream)
    size = tout[outl] - tin[outl] + 1
    big = outl[np.argsort(-size, kind="stable")[:384]]
    rng = np.random.default_rng(seed)
    rest = np.setdiff1d(outl, big)
    other = rng.choice(rest, size=min(128, rest.size), replace=False)
    interior = np.setdiff1d(np.arange(region.ncell), outl)
    inner = rng.choice(interior, size=256, replace=False)
    return np.unique(np.concatenate([big, other, inner])).astype(np.int32)


def regen_sample(region, every):
    if every is None:
        return np.arange(region.ncell, dtype=np.int32)
    a = region.arrays
    wb = (a["loc_lake"] > 0) | (a["loc_wetl"] > 0) | (a["glo_wetl"] > 0) | (a["glo_lake"] > 0) | \
         (a["glo_res"] > 0) | (a["lake_area"] > 0) | (a["res_area"] > 0)
    keep = wb.copy()
    keep[::every] = True
    return np.nonzero(keep)[0].astype(np.int32)


def regen_inputs(name):
    """(region, P, T, S, doy0, snapshot days, sampled cells, stations) of a regenerated case."""
    fac, nd, doy0, seed, snaps, every, kind = REGEN_CASES[name]
    region = getattr(sy, fac)()
    P, T, S = sy.forcing(region, nd, seed=seed, doy0=doy0)
    return region, P, T, S, doy0, snaps, regen_sample(region, every), regen_stations(region, kind)


def main_regen(names=None):
    from helpers import field_sums, input_digest
    if not ref_case.available():
        if not ref_case.build(REF_SOURCE):
            raise SystemExit("reference sources not found; cannot regenerate fixtures")
    for name in REGEN_CASES:
        if names and name not in names:
            continue
        region, P, T, S, doy0, snaps, sample, stations = regen_inputs(name)
        res = ref_case.run(region, P, T, S, doy0=doy0, stations=stations, snapshots=snaps)
        rep = ref_case.REF_BANDS // region.nband
        out = dict(digest=np.array(input_digest(region, P, T, S)), stations=res["stations"],
                   snap_days=np.array(snaps), discharge=res["discharge"], sample=sample,
                   keys=np.array(REGEN_KEYS))
        for i, snap in enumerate(res["snapshots"]):
            bands = snap.pop("snow_band").reshape(region.ncell, region.nband, rep)
            assert np.array_equal(bands, np.repeat(bands[:, :, :1], rep, axis=2))
            snap["snow_band"] = bands[:, :, 0].copy()
            out[f"s{i}_sums"] = field_sums(snap, REGEN_KEYS + ["snow_band"])
            if i == len(snaps) - 1:
                for k in REGEN_KEYS + ["snow_band", "k_release"]:
                    out[f"s{i}_{k}"] = snap[k][sample]
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{name}: {region.ncell} cells x {P.shape[0]} days, {sample.size} sampled cells, "
              f"{len(stations)} stations -> {os.path.getsize(path) / 1e6:.2f} MB")


if __name__ == "__main__":
    main_regen(sys.argv[1:])
    main(sys.argv[1:])
    main_wtemp(sys.argv[1:])
    main_wuse(sys.argv[1:])
    main_wuse_glwd(sys.argv[1:])
    main_outputs(sys.argv[1:])
    main_outputs_wuse(sys.argv[1:])
    main_outputs_wuse(sys.argv[1:], name="swb_outputs_glwd_730d", glwd=True)
    main_outputs_wtemp(sys.argv[1:])
    main_wtemp_wuse(sys.argv[1:])
