"""In-memory description of a simulated region (the static inputs of the daily step).

A ``Region`` carries, per land cell, what the reference keeps in its global
grids (``geo``, ``land``, ``GW``, ``maxSoilWaterCap``, ``calibParam`` and the
routing inputs of ``routingClass::init``, source/routing.cpp:131-742), in the
reference's storage types.  The GPU library receives it through the C ABI
(``include/wg_gpu.h``, struct ``wg_region``) without copying on the host.

Calibration parameters are held as one ``[NPARAM, ncell]`` float64 block in
the order of ``eCalibParam`` (source/calib_param.h:72-101).
"""
from __future__ import annotations

import dataclasses
from typing import Dict

import numpy as np

# eCalibParam order (source/calib_param.h:72-101)
PARAM_NAMES = (
    "P_GAMRUN_C", "P_CFA", "P_CFS", "M_ROOT_D", "M_RIVRGH_C", "P_LAK_D", "P_WET_D",
    "P_SWOUTF_C", "M_EVAREDEX", "M_NETRAD", "P_PTC_HUM", "P_PTC_ARI", "P_PET_MXDY",
    "P_MCWH", "M_LAI", "P_T_SNOWFZ", "P_T_SNOWMT", "M_DEGDAY_F", "P_T_GRADNT", "M_GW_F",
    "M_RG_MAX", "P_PCRITGWA", "P_GWOUTF_C", "M_NETABSSW", "M_NETABSGW", "M_PREC",
)
PARAM = {name: i for i, name in enumerate(PARAM_NAMES)}
NPARAM = len(PARAM_NAMES)

# JSON keys of the reference's parameter file (source/calib_param.h:131-222)
PARAM_JSON_KEYS = (
    "gammaHBV_runoff_coeff", "CFA_cellCorrFactor", "CFS_statCorrFactor", "root_depth_multiplier",
    "river_roughness_coeff_mult", "lake_depth", "wetland_depth", "surfacewater_outflow_coefficient",
    "evapo_red_fact_exp_mult", "net_radiation_mult", "PT_coeff_humid", "PT_coeff_arid",
    "max_daily_PET", "mcwh", "LAI_mult", "snow_freeze_temp", "snow_melt_temp",
    "degree_day_factor_mult", "temperature_gradient", "gw_factor_mult", "rg_max_mult",
    "pcrit_aridgw", "groundwater_outflow_coeff", "net_abstraction_surfacewater_mult",
    "net_abstraction_groundwater_mult", "precip_mult",
)

NLCT = 18

# (field, dtype, per) -- per: "cell", "band" (ncell*(nband+1)), "lct", "param"
FIELDS = (
    ("lct_albedo", np.float64, "lct"),
    ("lct_albedo_snow", np.float64, "lct"),
    ("lct_ddf", np.float64, "lct"),
    ("lct_lai_a", np.float32, "lct"),
    ("lct_lai_b", np.float32, "lct"),
    ("lct_initial_days", np.int16, "lct"),
    ("area_km2", np.float64, "cell"),
    ("lat_deg", np.float64, "cell"),
    ("contfreq", np.float64, "cell"),
    ("lct", np.uint8, "cell"),
    ("built_up", np.float32, "cell"),
    ("smax", np.float32, "cell"),
    ("lai_max", np.float32, "cell"),
    ("gw_factor", np.float32, "cell"),
    ("rg_max", np.int16, "cell"),
    ("texture", np.int8, "cell"),
    ("ldd", np.int8, "cell"),
    ("aindex", np.int16, "cell"),
    ("elev", np.int16, "band"),
    ("param", np.float64, "param"),
    ("loc_lake", np.float64, "cell"),
    ("loc_wetl", np.float64, "cell"),
    ("glo_wetl", np.float64, "cell"),
    ("glo_lake", np.float64, "cell"),
    ("glo_res", np.float64, "cell"),
    ("lake_area", np.float64, "cell"),
    ("res_area", np.float64, "cell"),
    ("stor_cap", np.float64, "cell"),
    ("mean_outflow", np.float64, "cell"),
    ("mean_demand", np.float64, "cell"),
    ("res_type", np.int8, "cell"),
    ("start_month", np.int8, "cell"),
    ("river_length", np.float64, "cell"),
    ("river_slope", np.float64, "cell"),
    ("roughness", np.float64, "cell"),
    ("bankfull", np.float64, "cell"),
    ("downstream", np.int32, "cell"),
    ("rout_order", np.int32, "cell"),
)


@dataclasses.dataclass
class Region:
    """Static inputs of one region; arrays are contiguous and typed as in FIELDS."""

    ncell: int
    nband: int
    arrays: Dict[str, np.ndarray]
    river_velo_opt: int = 1
    default_velocity: float = 86.4   # routingClass::routingClass, routing.cpp:119-122
    # options.fractionalRoutingOpt: part of the local runoff bypasses the cell's
    # water bodies and flows directly into its river (routing.cpp:1895-2046, 3408-3412)
    frac_routing: int = 0
    # options.statcorrOpt: each cell's outflow multiplied by its station correction
    # factor, the calibration parameter P_CFS (routing.cpp:3929-3931)
    statcorr_opt: int = 0
    # grid placement, used by the fixture writers (0.5-degree rows/cols, 1-based)
    row: np.ndarray | None = None
    col: np.ndarray | None = None
    name: str = ""

    def __post_init__(self):
        for fname, dt, per in FIELDS:
            a = self.arrays[fname]
            want = {"cell": (self.ncell,), "lct": (NLCT,), "band": (self.ncell * (self.nband + 1),),
                    "param": (NPARAM * self.ncell,)}[per]
            a = np.ascontiguousarray(a, dtype=dt).reshape(want)
            self.arrays[fname] = a

    def __getattr__(self, key):
        arrays = self.__dict__.get("arrays")
        if arrays is not None and key in arrays:
            return arrays[key]
        raise AttributeError(key)

    def param(self, name: str) -> np.ndarray:
        return self.arrays["param"].reshape(NPARAM, self.ncell)[PARAM[name]]

    def with_options(self, **kw) -> "Region":
        """The same region with dataclass fields replaced (e.g. frac_routing=1)."""
        out = dataclasses.replace(self, **kw)
        for k in ("lct_tables", "extras"):
            if k in self.__dict__:
                out.__dict__[k] = self.__dict__[k]
        return out

    def with_param(self, name: str, values) -> "Region":
        """The same region with calibration parameter ``name`` replaced (per cell)."""
        arrays = dict(self.arrays)
        p = self.arrays["param"].copy()
        p.reshape(NPARAM, self.ncell)[PARAM[name]] = values
        arrays["param"] = p
        out = dataclasses.replace(self, arrays=arrays)
        for k in ("lct_tables", "extras"):
            if k in self.__dict__:
                out.__dict__[k] = self.__dict__[k]
        return out

    def with_bands(self, nband: int) -> "Region":
        """The same region with each band replicated so that the total band count is
        ``nband`` (a multiple of the current count); band order stays ascending."""
        if nband % self.nband:
            raise ValueError("band count must be a multiple of the current one")
        rep = nband // self.nband
        e = self.arrays["elev"].reshape(self.ncell, self.nband + 1)
        e2 = np.concatenate([e[:, :1], np.repeat(e[:, 1:], rep, axis=1)], axis=1)
        arrays = dict(self.arrays)
        arrays["elev"] = e2.reshape(-1)
        out = dataclasses.replace(self, nband=nband, arrays=arrays)
        for k in ("lct_tables", "extras"):
            if k in self.__dict__:
                out.__dict__[k] = self.__dict__[k]
        return out

    def subset_order_check(self) -> None:
        """Raise if rout_order is not a topological order of downstream."""
        pos = np.empty(self.ncell, np.int64)
        pos[self.rout_order] = np.arange(self.ncell)
        d = self.downstream
        m = d >= 0
        if np.any(pos[d[m]] <= pos[np.nonzero(m)[0]]):
            raise ValueError("rout_order is not upstream-first")


STATE_FIELDS = (
    ("canopy", np.float64, "cell"), ("soil", np.float64, "cell"), ("snow", np.float64, "cell"),
    ("snow_band", np.float64, "bandstate"),
    ("lai_days", np.int32, "cell"), ("lai_status", np.int32, "cell"), ("lai_precsum", np.float64, "cell"),
    ("gw", np.float64, "cell"), ("river", np.float64, "cell"), ("loclake", np.float64, "cell"),
    ("locwetl", np.float64, "cell"), ("glolake", np.float64, "cell"), ("glowetl", np.float64, "cell"),
    ("res", np.float64, "cell"),
    ("rf_loclake", np.float64, "cell"), ("rf_locwetl", np.float64, "cell"), ("rf_glolake", np.float64, "cell"),
    ("rf_glowetl", np.float64, "cell"), ("rf_res", np.float64, "cell"),
    ("k_release", np.float64, "cell"),
    ("laf", np.float64, "cell"), ("laf_prev", np.float64, "cell"), ("fswb_next", np.float64, "cell"),
    ("laf_started", np.int32, "cell"),
)
STATE_NAMES = tuple(f for f, _, _ in STATE_FIELDS)


def empty_state(ncell: int, nband: int) -> Dict[str, np.ndarray]:
    out = {}
    for f, dt, per in STATE_FIELDS:
        out[f] = np.zeros(ncell * nband if per == "bandstate" else ncell, dt)
    return out


def save_npz(region: Region, path: str, **extra) -> None:
    """Store a region (and optional extra arrays) in one compressed .npz file."""
    payload = {f"a_{k}": v for k, v in region.arrays.items()}
    meta = np.array([region.ncell, region.nband, region.river_velo_opt, region.frac_routing, region.statcorr_opt],
                    np.int64)
    payload.update(meta=meta, default_velocity=np.array(region.default_velocity), name=np.array(region.name))
    if region.row is not None:
        payload.update(row=region.row, col=region.col)
    for k, v in getattr(region, "lct_tables", {}).items():
        payload[f"t_{k}"] = v
    for k, v in getattr(region, "extras", {}).items():
        payload[f"x_{k}"] = v
    for k, v in extra.items():
        payload[f"e_{k}"] = v
    np.savez_compressed(path, **payload)


def load_npz(path: str):
    """Inverse of save_npz: returns (region, extra_dict)."""
    z = np.load(path, allow_pickle=False)
    arrays = {k[2:]: z[k] for k in z.files if k.startswith("a_")}
    meta = [int(x) for x in z["meta"]]
    ncell, nband, velo = meta[:3]
    frac = meta[3] if len(meta) > 3 else 0
    statcorr = meta[4] if len(meta) > 4 else 0
    reg = Region(ncell=ncell, nband=nband, arrays=arrays, river_velo_opt=velo, frac_routing=frac, statcorr_opt=statcorr,
                 default_velocity=float(z["default_velocity"]), name=str(z["name"]),
                 row=z["row"] if "row" in z.files else None, col=z["col"] if "col" in z.files else None)
    reg.lct_tables = {k[2:]: z[k] for k in z.files if k.startswith("t_")}
    reg.extras = {k[2:]: z[k] for k in z.files if k.startswith("x_")}
    extra = {k[2:]: z[k] for k in z.files if k.startswith("e_")}
    return reg, extra


def inflow_cells(region) -> np.ndarray:
    """The cells flowing into each cell by direction, [ncell, 9] int32 (0-based,
    -1 none), the table the reference's water temperature reads
    (G_inflow_cells, built by rout_prepare.cpp:358-420): direction
    3 * (1 - drow) + (1 + dcol) of the upstream cell's offset, [4] the cell
    itself (never an inflow).  An upstream cell that is not a grid neighbour
    takes the first free direction."""
    n = region.ncell
    out = np.full((n, 9), -1, np.int32)
    down = region.downstream
    for m in np.nonzero(down >= 0)[0]:
        c = int(down[m])
        k = -1
        if region.row is not None:
            drow, dcol = int(region.row[m]) - int(region.row[c]), int(region.col[m]) - int(region.col[c])
            if abs(drow) <= 1 and abs(dcol) <= 1 and (drow, dcol) != (0, 0):
                k = 3 * (1 - drow) + (1 + dcol)
        if k < 0 or out[c, k] >= 0:
            free = [j for j in range(9) if j != 4 and out[c, j] < 0]
            if not free:
                raise ValueError(f"cell {c} has more than 8 upstream cells")
            k = free[0]
        out[c, k] = m
    return out


_FIRST_DAY_OF_MONTH = np.array([1, 32, 60, 91, 121, 152, 182, 213, 244, 274, 305, 335])


def use_rows(doy0: int, ndays: int) -> np.ndarray:
    """Row of the water-use tables for each day of a run that starts on day of
    year doy0: 12 x (years since the first day) + month, a new year starting at
    every day 1 after the first day (the reference reads one year's net uses at
    each year start, integrateWGHM.cpp:645-646)."""
    doy = (doy0 - 1 + np.arange(ndays)) % 365 + 1
    year = np.cumsum(np.r_[0, (doy[1:] == 1).astype(np.int64)])
    month = np.searchsorted(_FIRST_DAY_OF_MONTH, doy, side="right") - 1
    return (12 * year + month).astype(np.int64)


def year_spans(doy0: int, ndays: int) -> list:
    """The run's days split at year starts: [(first day index, days, day of year
    of the first day, year index)]."""
    out, d, doy, k = [], 0, int(doy0), 0
    while d < ndays:
        m = min(ndays - d, 365 - doy + 1)
        out.append((d, m, doy, k))
        d += m
        doy, k = 1, k + 1
    return out
