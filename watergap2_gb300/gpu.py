"""ctypes binding of the C ABI of ``_build/libwg_gpu.so`` (include/wg_gpu.h).

``Model`` mirrors the reference's pair of day-step objects for one region on one
GB300: ``step_vertical`` is the whole-grid counterpart of
``dailyWaterBalanceClass::calcNewDay`` (source/daily.h:24), ``step_routing`` of
``routingClass::routing`` + ``updateLandAreaFrac`` (source/routing.h:44-46), and
``run_days`` runs many days in one persistent launch.  There is no CPU fallback:
if the library or a GPU is missing, construction raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .region import FIELDS, STATE_FIELDS, Region, empty_state

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libwg_gpu.so")

WG_OK = 0
WU_NSTATE = 13   # WG_WU_NSTATE: rows of the water-use state
STATUS = {0: "ok", 1: "invalid argument", 2: "unsupported option", 3: "CUDA error", 4: "out of device memory",
          5: "invalid drainage topology", 6: "device wait exceeded its limit", 7: "no usable device"}

# exported entry points of include/wg_gpu.h
SYMBOLS = ("wg_create", "wg_destroy", "wg_set_state", "wg_get_state", "wg_set_member_state",
           "wg_get_member_state", "wg_upload_forcing", "wg_step_vertical", "wg_step_routing", "wg_run_days",
           "wg_get_discharge", "wg_get_balance", "wg_reset_balance", "wg_synchronize", "wg_launch_shape",
           "wg_get_launch_shape", "wg_num_levels", "wg_launch_count", "wg_last_error", "wg_status_string",
           "wg_measure_fp64_peak", "wg_run_steps", "wg_run_num_steps", "wg_get_balance_noalloc",
           "wg_set_chunk_steps", "wg_get_chunk_steps", "wg_set_vertical_overlap", "wg_get_vertical_overlap",
           "wg_math_eval", "wg_upload_longwave", "wg_set_water_temp_inputs", "wg_get_water_temp",
           "wg_set_water_temp", "wg_get_river_temp", "wg_clear_error", "wg_set_barrier_test", "wg_autotune", "wg_graph_capture", "wg_graph_launch",
           "wg_set_calib_param", "wg_save_snapshot", "wg_restore_snapshot", "wg_kernel_timing",
           "wg_get_kernel_times", "wg_set_member_factors", "wg_upload_forcing_async", "wg_set_active_cells",
           "wg_upload_forcing_unf", "wg_read_unf", "wg_monthly_outputs", "wg_get_monthly", "wg_set_step_sync",
           "wg_upload_water_use", "wg_set_water_use_inputs", "wg_get_water_use", "wg_set_water_use",
           "wg_model_options_default", "wg_get_member_discharge", "wg_set_deferred",
           "wg_record_daily_storages", "wg_get_daily_storages", "wg_upload_forcing_cells",
           "wg_monthly_outputs_vertical", "wg_daily_outputs_vertical", "wg_get_daily_vertical",
           "wg_monthly_outputs_routing", "wg_daily_outputs_routing", "wg_get_daily_routing")


class WgError(RuntimeError):
    pass


class _Region(ctypes.Structure):
    _fields_ = [("ncell", ctypes.c_int32), ("nband", ctypes.c_int32), ("river_velo_opt", ctypes.c_int32),
                ("frac_routing", ctypes.c_int32), ("default_velocity", ctypes.c_double)] + \
               [(name, ctypes.c_void_p) for name, _, _ in FIELDS] + [("glwd_unit", ctypes.c_void_p),
                                                                      ("lct_kc_min", ctypes.c_void_p),
                                                                      ("lct_kc_max", ctypes.c_void_p)]


class _StateView(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name, _, _ in STATE_FIELDS]


class _TuneResult(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int32), ("blocks", ctypes.c_int32), ("chunk_steps", ctypes.c_int32),
                ("trials", ctypes.c_int32), ("ms_per_step", ctypes.c_double)]


class _Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("max_days", ctypes.c_int32), ("nstation", ctypes.c_int32),
                ("record_balance", ctypes.c_int32), ("stations", ctypes.c_void_p), ("stream", ctypes.c_uint64),
                ("precision", ctypes.c_int32), ("members", ctypes.c_int32), ("member_prec_factor", ctypes.c_void_p),
                ("member_gamma_factor", ctypes.c_void_p), ("block_threads", ctypes.c_int32),
                ("ring_days", ctypes.c_int32), ("days_per_step", ctypes.c_int32), ("water_temp", ctypes.c_int32),
                ("water_use", ctypes.c_int32), ("model", ctypes.c_void_p)]


# wg_model_options: the reference's model switches (optionClass, option.h:43-68)
MODEL_OPTIONS = ("time_series", "cloud", "intercept", "calc_albedo", "use_kc", "pet_opt", "clcl_opt", "perma_opt",
                 "glacier_opt", "land_cover_opt", "arid_area_opt", "river_evapo_opt", "statcorr_opt", "use_alloc",
                 "aggr_nus_glo_lak_res_opt", "ant_nat_opt", "res_year_opt", "res_opt",
                 "climate_spatial_resolution")


class _ModelOptions(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int32) for f in MODEL_OPTIONS]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise WgError(f"{path} is missing: build it with watergap2_gb300.build.build()")
    lib = ctypes.CDLL(path)
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    lib.wg_create.argtypes = [ctypes.POINTER(_Region), ctypes.POINTER(_Options), ctypes.POINTER(vp)]
    lib.wg_model_options_default.argtypes = [ctypes.POINTER(_ModelOptions)]
    lib.wg_model_options_default.restype = None
    lib.wg_destroy.argtypes = [vp]
    lib.wg_set_state.argtypes = [vp, ctypes.POINTER(_StateView)]
    lib.wg_get_state.argtypes = [vp, ctypes.POINTER(_StateView)]
    lib.wg_set_member_state.argtypes = [vp, i32, ctypes.POINTER(_StateView)]
    lib.wg_get_member_state.argtypes = [vp, i32, ctypes.POINTER(_StateView)]
    lib.wg_launch_shape.argtypes = [vp, i32, i32]
    lib.wg_get_launch_shape.argtypes = [vp, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(i32)]
    lib.wg_upload_forcing.argtypes = [vp, i32, i32, vp, vp, vp]
    lib.wg_upload_forcing_async.argtypes = [vp, i32, i32, vp, vp, vp]
    lib.wg_step_vertical.argtypes = [vp, i32, i32]
    lib.wg_step_routing.argtypes = [vp, i32, i32]
    lib.wg_run_days.argtypes = [vp, i32, i32, i32]
    lib.wg_run_steps.argtypes = [vp, i32, i32, i32, i32, i32]
    lib.wg_run_steps.restype = ctypes.c_int
    lib.wg_run_num_steps.argtypes = [vp, i32]
    lib.wg_run_num_steps.restype = i32
    lib.wg_get_discharge.argtypes = [vp, i32, i32, vp]
    lib.wg_get_member_discharge.argtypes = [vp, i32, i32, i32, vp]
    lib.wg_set_deferred.argtypes = [vp, i32]
    lib.wg_upload_forcing_cells.argtypes = [vp, i32, i32, i32, i32, vp, vp, vp, i32]
    lib.wg_record_daily_storages.argtypes = [vp, i32]
    lib.wg_get_daily_storages.argtypes = [vp, i32, i32, vp]
    lib.wg_get_balance.argtypes = [vp, vp]
    lib.wg_reset_balance.argtypes = [vp]
    lib.wg_get_balance_noalloc.argtypes = [vp, vp]
    lib.wg_get_balance_noalloc.restype = ctypes.c_int
    lib.wg_synchronize.argtypes = [vp]
    lib.wg_num_levels.argtypes = [vp]
    lib.wg_num_levels.restype = i32
    lib.wg_launch_count.argtypes = [vp]
    lib.wg_launch_count.restype = i64
    lib.wg_last_error.argtypes = [vp]
    lib.wg_last_error.restype = ctypes.c_char_p
    lib.wg_measure_fp64_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.wg_measure_fp64_peak.restype = ctypes.c_int
    lib.wg_kernel_timing.argtypes = [vp, i32]
    lib.wg_get_kernel_times.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(i32)]
    lib.wg_set_calib_param.argtypes = [vp, i32, vp]
    lib.wg_set_member_factors.argtypes = [vp, vp, vp]
    lib.wg_set_active_cells.argtypes = [vp, vp]
    lib.wg_upload_forcing_unf.argtypes = [vp, i32, i32, i32, i32, vp, vp, vp, i32]
    lib.wg_monthly_outputs.argtypes = [vp, i32, i32]
    lib.wg_monthly_outputs_vertical.argtypes = [vp, i32]
    lib.wg_monthly_outputs_vertical.restype = i32
    lib.wg_daily_outputs_vertical.argtypes = [vp, i32]
    lib.wg_daily_outputs_vertical.restype = i32
    lib.wg_get_daily_vertical.argtypes = [vp, i32, i32, i32, vp]
    lib.wg_get_daily_vertical.restype = i32
    lib.wg_monthly_outputs_routing.argtypes = [vp, i32]
    lib.wg_monthly_outputs_routing.restype = i32
    lib.wg_daily_outputs_routing.argtypes = [vp, i32]
    lib.wg_daily_outputs_routing.restype = i32
    lib.wg_get_daily_routing.argtypes = [vp, i32, i32, i32, vp]
    lib.wg_get_daily_routing.restype = i32
    lib.wg_set_step_sync.argtypes = [vp, i32]
    lib.wg_get_monthly.argtypes = [vp, i32, i32, i32, vp]
    lib.wg_read_unf.argtypes = [ctypes.c_char_p, vp, i64]
    lib.wg_read_unf.restype = i64
    lib.wg_save_snapshot.argtypes = [vp]
    lib.wg_restore_snapshot.argtypes = [vp]
    lib.wg_set_chunk_steps.argtypes = [vp, i32]
    lib.wg_get_chunk_steps.argtypes = [vp]
    lib.wg_get_chunk_steps.restype = i32
    lib.wg_math_eval.argtypes = [i32, i32, vp, vp, ctypes.c_int64, vp]
    lib.wg_upload_longwave.argtypes = [vp, i32, i32, vp]
    lib.wg_upload_water_use.argtypes = [vp, i32, i32, i32, vp, vp, vp, vp]
    lib.wg_set_water_use_inputs.argtypes = [vp, vp]
    lib.wg_get_water_use.argtypes = [vp, vp]
    lib.wg_set_water_use.argtypes = [vp, vp]
    lib.wg_set_water_temp_inputs.argtypes = [vp, vp, vp]
    lib.wg_get_water_temp.argtypes = [vp, vp, vp]
    lib.wg_set_water_temp.argtypes = [vp, vp, vp]
    lib.wg_get_river_temp.argtypes = [vp, i32, i32, vp]
    lib.wg_clear_error.argtypes = [vp]
    lib.wg_set_barrier_test.argtypes = [vp, i32]
    lib.wg_set_vertical_overlap.argtypes = [vp, i32]
    lib.wg_get_vertical_overlap.argtypes = [vp]
    lib.wg_get_vertical_overlap.restype = i32
    lib.wg_autotune.argtypes = [vp, i32, i32, i32, i32, i32, ctypes.POINTER(_TuneResult)]
    lib.wg_graph_capture.argtypes = [vp, i32, i32, i32, i32, i32]
    lib.wg_graph_launch.argtypes = [vp]
    lib.wg_status_string.argtypes = [ctypes.c_int]
    lib.wg_status_string.restype = ctypes.c_char_p
    for name in ("wg_create", "wg_destroy", "wg_set_state", "wg_get_state", "wg_set_member_state",
                 "wg_get_member_state", "wg_upload_forcing", "wg_step_vertical", "wg_step_routing", "wg_run_days",
                 "wg_get_discharge", "wg_get_balance", "wg_reset_balance", "wg_synchronize", "wg_launch_shape",
                 "wg_get_launch_shape", "wg_set_chunk_steps", "wg_autotune", "wg_graph_capture", "wg_graph_launch",
                 "wg_set_calib_param", "wg_save_snapshot", "wg_restore_snapshot", "wg_kernel_timing",
                 "wg_get_kernel_times", "wg_set_member_factors", "wg_upload_forcing_async",
                 "wg_set_active_cells", "wg_upload_forcing_unf", "wg_monthly_outputs", "wg_get_monthly",
                 "wg_set_step_sync", "wg_set_vertical_overlap", "wg_upload_longwave", "wg_set_water_temp_inputs",
                 "wg_get_water_temp", "wg_set_water_temp", "wg_get_river_temp", "wg_clear_error",
                 "wg_set_barrier_test", "wg_upload_water_use", "wg_set_water_use_inputs", "wg_get_water_use",
                 "wg_set_water_use"):
        getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


def read_unf(path: str, nbytes: int, out: np.ndarray | None = None) -> np.ndarray:
    """wg_read_unf: nbytes of a file into out (uint8, e.g. pinned), or a new array."""
    lib = load_library()
    buf = np.empty(nbytes, np.uint8) if out is None else out
    assert buf.nbytes >= nbytes and buf.flags.c_contiguous
    got = lib.wg_read_unf(path.encode(), buf.ctypes.data, int(nbytes))
    if got != nbytes:
        raise WgError(f"wg_read_unf {path}: read {got} of {nbytes} bytes")
    return buf


MATH_FN = {"exp": 0, "log": 1, "pow": 2, "rcp": 3, "rcp_approx": 4}


def math_eval(fn: str, x, y=None, device: int = 0) -> np.ndarray:
    """wg_math_eval: the FP64 path's own exp / log / pow / reciprocal on the device."""
    lib = load_library()
    x = np.ascontiguousarray(x, np.float64)
    yy = None if y is None else np.ascontiguousarray(np.broadcast_to(y, x.shape), np.float64)
    out = np.empty_like(x)
    rc = lib.wg_math_eval(int(device), MATH_FN[fn], x.ctypes.data, None if yy is None else yy.ctypes.data,
                          int(x.size), out.ctypes.data)
    if rc != WG_OK:
        raise WgError(f"wg_math_eval: {STATUS.get(rc, rc)}")
    return out


def measure_fp64_peak(device: int = 0) -> float:
    """FP64 FMA throughput of the device in TFLOP/s (a dependent-chain-free DFMA loop)."""
    lib = load_library()
    v = ctypes.c_double(0.0)
    rc = lib.wg_measure_fp64_peak(int(device), ctypes.byref(v))
    if rc != WG_OK:
        raise WgError(f"wg_measure_fp64_peak: {STATUS.get(rc, rc)}")
    return float(v.value)


def _ptr(a):
    return a.ctypes.data if a is not None else None


class Model:
    """One region resident on one GPU."""

    def __init__(self, region: Region, max_days: int = 366, stations=None, record_balance: bool = False,
                 device: int = 0, stream: int = 0, precision: str = "fp64", members: int = 1,
                 prec_factor=None, gamma_factor=None, block_threads: int = 0, ring_days: int = 0,
                 days_per_step: int = 0, water_temp: bool = False, water_use: int | bool = False,
                 model_options: dict | None = None, glwd_unit=None):
        self.lib = load_library()
        self.region = region
        self._keep = []
        self._inflight = []
        r = _Region()
        r.ncell, r.nband, r.river_velo_opt = region.ncell, region.nband, region.river_velo_opt
        r.default_velocity = region.default_velocity
        r.frac_routing = int(getattr(region, "frac_routing", 0))
        for name, _, _ in FIELDS:
            a = region.arrays[name]
            self._keep.append(a)
            setattr(r, name, a.ctypes.data)
        # GLWD units (G_glwdUnit): with water use, the riparian cells' net abstractions
        # are met by their global lake's or reservoir's outflow cell (aggrNUsGloLakResOpt = 1)
        if glwd_unit is not None:
            u = np.ascontiguousarray(glwd_unit, np.int32)
            if u.shape != (region.ncell,):
                raise ValueError("glwd_unit is one unit per cell")
            self._keep.append(u)
            r.glwd_unit = u.ctypes.data
        # the land covers' crop coefficients (LAI_22.DAT), for the daily grids' Kc
        tabs = getattr(region, "lct_tables", None) or {}
        if "kc_min" in tabs and "kc_max" in tabs:
            for name in ("kc_min", "kc_max"):
                t = np.ascontiguousarray(tabs[name], np.float64)
                self._keep.append(t)
                setattr(r, "lct_" + name, t.ctypes.data)
        self.stations = np.ascontiguousarray(
            np.nonzero(region.downstream < 0)[0] if stations is None else stations, np.int32)
        o = _Options()
        o.device, o.max_days, o.nstation = device, int(max_days), int(self.stations.size)
        o.record_balance = int(bool(record_balance))
        o.stations = self.stations.ctypes.data
        o.stream = int(stream)
        o.precision = {"fp64": 0, "fp32": 1}[precision]
        o.members = int(members)
        self.members = int(members)
        self.precision = precision
        self._pf = None if prec_factor is None else np.ascontiguousarray(prec_factor, np.float32)
        self._gf = None if gamma_factor is None else np.ascontiguousarray(gamma_factor, np.float32)
        o.member_prec_factor = self._pf.ctypes.data if self._pf is not None else None
        o.member_gamma_factor = self._gf.ctypes.data if self._gf is not None else None
        o.block_threads = int(block_threads)
        o.ring_days = int(ring_days)
        o.days_per_step = int(days_per_step)
        o.water_temp = int(bool(water_temp))
        o.water_use = int(water_use)   # True/1; 2: delayed satisfaction
        # the reference's model switches: the built defaults, the region's station
        # correction, then the caller's values (refused by wg_create if not built)
        self._model = _ModelOptions()
        self.lib.wg_model_options_default(ctypes.byref(self._model))
        self._model.statcorr_opt = int(getattr(region, "statcorr_opt", 0))
        self._model.aggr_nus_glo_lak_res_opt = int(glwd_unit is not None)
        for k, v in (model_options or {}).items():
            if k not in MODEL_OPTIONS:
                raise WgError(f"unknown model option {k}")
            setattr(self._model, k, int(v))
        o.model = ctypes.addressof(self._model)
        self.max_days = int(max_days)
        h = ctypes.c_void_p()
        self._check(self.lib.wg_create(ctypes.byref(r), ctypes.byref(o), ctypes.byref(h)), "wg_create", None)
        self.h = h

    def _check(self, rc, what, h="self"):
        if rc != WG_OK:
            msg = ""
            if h is not None and getattr(self, "h", None):
                msg = self.lib.wg_last_error(self.h).decode()
            elif h is None:   # wg_create: the calling thread's reason
                msg = self.lib.wg_last_error(None).decode()
            raise WgError(f"{what}: {STATUS.get(rc, rc)} {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.wg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_levels(self) -> int:
        return int(self.lib.wg_num_levels(self.h))

    @property
    def launch_count(self) -> int:
        return int(self.lib.wg_launch_count(self.h))

    def upload_forcing(self, day0: int, P, T, S, overlap: bool = False):
        """Forcing of len(P) days into day slots day0..; with overlap, on the copy
        stream alongside runs in flight (wg_upload_forcing_async: the days written
        must not be read by those runs; pinned sources stay unchanged until the
        next synchronize).  A variable given as None keeps the slots' values."""
        P, T, S = (None if x is None else np.ascontiguousarray(x, np.float32) for x in (P, T, S))
        nd = next(x for x in (P, T, S) if x is not None).shape[0]
        fn = self.lib.wg_upload_forcing_async if overlap else self.lib.wg_upload_forcing
        if overlap:
            self._inflight.append((P, T, S))   # alive until the next synchronize
        self._check(fn(self.h, int(day0), nd, _ptr(P), _ptr(T), _ptr(S)), "upload_forcing")

    def upload_forcing_cells(self, day0: int, P, T, S, d_first: int = 0, ndays: int | None = None,
                             overlap: bool = False):
        """Cell-major float forcing [ncell, nd_file] (the reference's in-memory
        yearly grids) into day slots day0..: wg_upload_forcing_cells."""
        P, T, S = (np.ascontiguousarray(x, np.float32) for x in (P, T, S))
        nd_file = P.shape[1]
        ndays = nd_file - d_first if ndays is None else ndays
        if overlap:
            self._inflight.append((P, T, S))
        self._check(self.lib.wg_upload_forcing_cells(self.h, int(day0), nd_file, int(d_first), int(ndays), _ptr(P),
                                                     _ptr(T), _ptr(S), int(bool(overlap))), "upload_forcing_cells")

    def upload_forcing_unf(self, day0: int, prec_raw, temp_raw, swrad_raw, nd_file: int = 365, d_first: int = 0,
                           ndays: int | None = None, overlap: bool = False):
        """Days [d_first, d_first + ndays) of three raw `.365.UNF0` files (bytes as read,
        big-endian cell-major [ncell][nd_file]) into day slots day0.. ."""
        raws = [np.ascontiguousarray(np.frombuffer(r, np.uint8) if isinstance(r, (bytes, bytearray)) else r)
                for r in (prec_raw, temp_raw, swrad_raw)]
        for r in raws:
            assert r.nbytes == self.region.ncell * nd_file * 4, (r.nbytes, self.region.ncell * nd_file * 4)
        nd = nd_file - d_first if ndays is None else ndays
        if overlap:
            self._inflight.append(tuple(raws))
        self._check(self.lib.wg_upload_forcing_unf(self.h, int(day0), int(nd_file), int(d_first), int(nd),
                                                   _ptr(raws[0]), _ptr(raws[1]), _ptr(raws[2]), int(bool(overlap))),
                    "upload_forcing_unf")

    def step_vertical(self, doy: int, fday: int):
        self._check(self.lib.wg_step_vertical(self.h, int(doy), int(fday)), "step_vertical")

    def set_deferred(self, enable: bool = True):
        """wg_set_deferred: queue the per-day calls and run consecutive days as one
        day-pipelined run when a result is next needed."""
        self._check(self.lib.wg_set_deferred(self.h, int(bool(enable))), "set_deferred")

    def record_daily_storages(self, enable: bool = True):
        """wg_record_daily_storages: keep every cell's day-end routing storages."""
        self._check(self.lib.wg_record_daily_storages(self.h, int(bool(enable))), "record_daily_storages")

    def daily_storages(self, day0: int, ndays: int) -> np.ndarray:
        """[ndays, 7, ncell]: local lake, local wetland, global lake, global wetland,
        reservoir, river, groundwater [km3] after each output day."""
        out = np.zeros((ndays, 7, self.region.ncell))
        self._check(self.lib.wg_get_daily_storages(self.h, int(day0), int(ndays), _ptr(out)), "get_daily_storages")
        return out

    def step_routing(self, doy: int, oday: int):
        self._check(self.lib.wg_step_routing(self.h, int(doy), int(oday)), "step_routing")

    def run_days(self, doy0: int, fday0: int, ndays: int):
        self._check(self.lib.wg_run_days(self.h, int(doy0), int(fday0), int(ndays)), "run_days")

    def run_steps(self, doy0: int, fday0: int, ndays: int, t_begin: int, t_end: int):
        self._check(self.lib.wg_run_steps(self.h, int(doy0), int(fday0), int(ndays), int(t_begin), int(t_end)),
                    "run_steps")

    def num_steps(self, ndays: int) -> int:
        return int(self.lib.wg_run_num_steps(self.h, int(ndays)))

    def synchronize(self):
        self._check(self.lib.wg_synchronize(self.h), "synchronize")
        self._inflight.clear()

    def discharge(self, day0: int, ndays: int) -> np.ndarray:
        """[ndays, nstation] (single member) or [ndays, nstation, members]."""
        shape = (ndays, self.stations.size) if self.members == 1 else (ndays, self.stations.size, self.members)
        out = np.zeros(shape)
        self._check(self.lib.wg_get_discharge(self.h, int(day0), int(ndays), _ptr(out)), "get_discharge")
        return out

    def member_discharge(self, member: int, day0: int, ndays: int) -> np.ndarray:
        """Discharge of one ensemble member [ndays, nstation]."""
        out = np.zeros((ndays, self.stations.size))
        self._check(self.lib.wg_get_member_discharge(self.h, int(member), int(day0), int(ndays), _ptr(out)),
                    "get_member_discharge")
        return out

    def discharge_into(self, day0: int, ndays: int, out: np.ndarray) -> np.ndarray:
        """Like discharge() but into a caller-provided (e.g. pinned) float64 array."""
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size >= ndays * self.stations.size
        self._check(self.lib.wg_get_discharge(self.h, int(day0), int(ndays), _ptr(out)), "get_discharge")
        return out

    def balance(self) -> np.ndarray:
        out = np.zeros(6)
        self._check(self.lib.wg_get_balance(self.h, _ptr(out)), "get_balance")
        return out

    def balance_noalloc(self) -> np.ndarray:
        """wg_get_balance_noalloc: the balance sums without any device allocation."""
        out = np.zeros(6)
        self._check(self.lib.wg_get_balance_noalloc(self.h, _ptr(out)), "get_balance_noalloc")
        return out

    def reset_balance(self):
        self._check(self.lib.wg_reset_balance(self.h), "reset_balance")

    def get_state(self, member: int = 0, fields=None) -> dict:
        """The state in cell order; `fields` limits the copy to those fields."""
        st = empty_state(self.region.ncell, self.region.nband)
        if fields is not None:
            st = {k: a for k, a in st.items() if k in fields}
        v = _StateView()
        for k, a in st.items():
            setattr(v, k, a.ctypes.data)
        self._check(self.lib.wg_get_member_state(self.h, int(member), ctypes.byref(v)), "get_state")
        return st

    def set_state(self, st: dict, member: int = 0):
        v = _StateView()
        keep = []
        for name, dt, _ in STATE_FIELDS:
            a = np.ascontiguousarray(st[name], dt)
            keep.append(a)
            setattr(v, name, a.ctypes.data)
        self._check(self.lib.wg_set_member_state(self.h, int(member), ctypes.byref(v)), "set_state")

    def launch_shape(self, threads: int | None = None, blocks: int | None = None):
        """Set (threads, blocks) of the persistent kernels if given; return (threads, blocks, max_blocks)."""
        if threads is not None:
            self._check(self.lib.wg_launch_shape(self.h, int(threads), int(blocks or 0)), "launch_shape")
        t, b, mb = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._check(self.lib.wg_get_launch_shape(self.h, ctypes.byref(t), ctypes.byref(b), ctypes.byref(mb)),
                    "get_launch_shape")
        return t.value, b.value, mb.value

    def set_calib_param(self, name: str, values):
        """wg_set_calib_param for P_GAMRUN_C or P_CFA, values per cell."""
        k = {"P_GAMRUN_C": 0, "P_CFA": 1}[name]
        v = np.ascontiguousarray(values, np.float64)
        assert v.shape == (self.region.ncell,)
        self._check(self.lib.wg_set_calib_param(self.h, k, _ptr(v)), "set_calib_param")

    def vinline_fraction(self) -> float:
        """Fraction of cells whose vertical balance runs inside the wavefront (a water
        body, or no land outside the water bodies, or no continental area) -- the
        rule of wg_create, on the continental share as geo.init raises it to the
        lake and reservoir share (geo.cpp:25-45)."""
        r = self.region
        wb = (r.loc_lake > 0) | (r.loc_wetl > 0) | (r.lake_area > 0) | (r.res_area > 0) | (r.glo_wetl > 0)
        cf = np.maximum(r.contfreq, ((r.loc_lake + r.glo_lake) + 0.0) + r.glo_res)
        l0 = cf - (r.glo_lake + r.glo_wetl + r.loc_lake + r.loc_wetl + r.glo_res)
        return float(np.mean(wb | ~(l0 > 0) | (cf < 1e-6)))

    def kernel_timing(self, enable: bool = True):
        self._check(self.lib.wg_kernel_timing(self.h, int(bool(enable))), "kernel_timing")

    def kernel_times(self) -> dict:
        """Summed device ms of the vertical-ahead and wavefront launches since the last call."""
        a, b, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int32()
        self._check(self.lib.wg_get_kernel_times(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(n)),
                    "get_kernel_times")
        return {"vertical_ahead_ms": a.value, "wavefront_ms": b.value, "launch_pairs": n.value}

    def step_sync(self, flags: int):
        """wg_set_step_sync: 0 grid barrier per step, 1 per-warp step flags."""
        self._check(self.lib.wg_set_step_sync(self.h, int(flags)), "set_step_sync")

    MONTHLY = {"river_avail": 0, "storage": 1, "min_avail": 2, "max_avail": 3, "cell_runoff": 4, "velocity": 5}
    # the vertical balance's monthly grids (wg_monthly_outputs_vertical), which = 6 + index
    MONTHLY_VERTICAL = ["prec", "temp", "ext_rad", "short_up_rad", "short_down_rad", "net_short_rad", "net_long_rad",
                        "net_rad", "open_water_pet", "pet", "aet", "land_aet", "land_aet_uncorr", "lai", "albedo",
                        "interception", "canopy_wc", "max_canopy_wc", "snowfall", "rainfall", "snowmelt",
                        "snow_evap", "swe", "snow_cover", "soil_wc", "runoff", "urban_runoff", "surface_runoff",
                        "gw_recharge", "canopy_storage", "snow_storage", "soil_storage", "total_pet"]
    MONTHLY.update({k: 6 + i for i, k in enumerate(MONTHLY_VERTICAL)})
    # the vertical balance's daily grids (wg_daily_outputs_vertical), field = index
    DAILY_VERTICAL = ["prec", "temp", "pet", "total_pet", "lai", "kc", "albedo", "interception", "canopy_wc",
                      "max_canopy_wc", "snowfall", "snowmelt", "swe", "snow_cover", "soil_wc", "surface_runoff",
                      "gw_recharge", "ext_rad", "short_down_rad", "short_up_rad", "net_short_rad", "net_long_rad",
                      "net_rad", "canopy_storage", "snow_storage", "soil_storage", "land_aet"]
    # routing's further monthly grids (wg_monthly_outputs_routing), which = 39 + index,
    # and the cell AET grids assembled from both sets
    MONTHLY_ROUTING = ["open_water_evap", "cell_surface_runoff", "gw_runoff", "land_area_frac", "loc_wetl_extent",
                       "glo_wetl_extent", "res_inflow", "res_outflow", "consistent_precip", "surf_storage",
                       "actual_use", "nug"]
    MONTHLY.update({k: i for i, k in enumerate(MONTHLY_ROUTING, 6 + len(MONTHLY_VERTICAL))})
    MONTHLY.update({"cell_aet": 6 + len(MONTHLY_VERTICAL) + len(MONTHLY_ROUTING),
                    "cell_aet_wca": 7 + len(MONTHLY_VERTICAL) + len(MONTHLY_ROUTING)})
    # with the water temperature: the monthly mean temperatures (-9999 without a computed day)
    MONTHLY_WTEMP = ["wt_river", "wt_loclake", "wt_locwetl", "wt_glolake", "wt_res", "wt_glowetl"]
    MONTHLY.update({k: i for i, k in enumerate(MONTHLY_WTEMP, 8 + len(MONTHLY_VERTICAL) + len(MONTHLY_ROUTING))})
    # routing's daily grids (wg_daily_outputs_routing), field = index
    DAILY_ROUTING = ["river_avail", "velocity", "cell_runoff", "cell_runoff_mm", "cell_surface_runoff", "gw_runoff",
                     "land_area_frac", "consistent_precip", "open_water_evap", "cell_aet"]

    def monthly_outputs_routing(self, enable: bool = True):
        """wg_monthly_outputs_routing: routing's further monthly grids too."""
        self._check(self.lib.wg_monthly_outputs_routing(self.h, int(bool(enable))), "monthly_outputs_routing")

    def daily_outputs_routing(self, ndays: int):
        """wg_daily_outputs_routing: routing's daily grids for output days 0 .. ndays-1 (0: off)."""
        self._check(self.lib.wg_daily_outputs_routing(self.h, int(ndays)), "daily_outputs_routing")
        self.droute_days = int(ndays)

    def daily_routing(self, name: str, day0: int = 0, nd: int | None = None) -> np.ndarray:
        """[nd, ncell] daily routing grid, cell order."""
        nd = self.droute_days - day0 if nd is None else nd
        out = np.zeros((nd, self.region.ncell))
        self._check(self.lib.wg_get_daily_routing(self.h, self.DAILY_ROUTING.index(name), int(day0), int(nd),
                                                  _ptr(out)), "get_daily_routing")
        return out

    def daily_outputs_vertical(self, ndays: int):
        """wg_daily_outputs_vertical: the vertical balance's daily grids for output
        days 0 .. ndays-1 (0: off)."""
        self._check(self.lib.wg_daily_outputs_vertical(self.h, int(ndays)), "daily_outputs_vertical")
        self.daily_days = int(ndays)

    def daily_vertical(self, name: str, day0: int = 0, nd: int | None = None) -> np.ndarray:
        """[nd, ncell] daily grid, cell order."""
        nd = self.daily_days - day0 if nd is None else nd
        out = np.zeros((nd, self.region.ncell))
        self._check(self.lib.wg_get_daily_vertical(self.h, self.DAILY_VERTICAL.index(name), int(day0), int(nd),
                                                   _ptr(out)), "get_daily_vertical")
        return out

    def monthly_outputs(self, nmonths: int, doy_day0: int = 1):
        """wg_monthly_outputs: accumulate monthly aggregates for nmonths months."""
        self._check(self.lib.wg_monthly_outputs(self.h, int(nmonths), int(doy_day0)), "monthly_outputs")
        self.nmonths = int(nmonths)

    def monthly_outputs_vertical(self, enable: bool = True):
        """wg_monthly_outputs_vertical: the vertical balance's monthly grids too."""
        self._check(self.lib.wg_monthly_outputs_vertical(self.h, int(bool(enable))), "monthly_outputs_vertical")

    def monthly(self, name: str, m0: int = 0, nm: int | None = None) -> np.ndarray:
        """[nm, ncell] (or [nm, ncell, members]) monthly aggregate, cell order."""
        nm = self.nmonths - m0 if nm is None else nm
        out = np.zeros((nm, self.region.ncell) if self.members == 1 else (nm, self.region.ncell, self.members))
        self._check(self.lib.wg_get_monthly(self.h, self.MONTHLY[name], int(m0), int(nm), _ptr(out)), "get_monthly")
        return out

    def set_active_cells(self, active=None):
        """wg_set_active_cells: run only the cells where active is true (None: all)."""
        a = None if active is None else np.ascontiguousarray(np.asarray(active, bool).astype(np.uint8))
        assert a is None or a.shape == (self.region.ncell,)
        self._check(self.lib.wg_set_active_cells(self.h, _ptr(a)), "set_active_cells")

    def set_member_factors(self, prec_factor=None, gamma_factor=None):
        pf = None if prec_factor is None else np.ascontiguousarray(prec_factor, np.float32)
        gf = None if gamma_factor is None else np.ascontiguousarray(gamma_factor, np.float32)
        for a in (pf, gf):
            assert a is None or a.shape == (self.members,)
        self._check(self.lib.wg_set_member_factors(self.h, _ptr(pf), _ptr(gf)), "set_member_factors")

    def save_snapshot(self):
        self._check(self.lib.wg_save_snapshot(self.h), "save_snapshot")

    def restore_snapshot(self):
        self._check(self.lib.wg_restore_snapshot(self.h), "restore_snapshot")

    def chunk_steps(self, steps: int | None = None) -> int:
        """Set the wavefront steps per launch if given (0 = the default); return the value in use."""
        if steps is not None:
            self._check(self.lib.wg_set_chunk_steps(self.h, int(steps)), "set_chunk_steps")
        return int(self.lib.wg_get_chunk_steps(self.h))

    def clear_error(self):
        """wg_clear_error: accept results again after a device-side wait ran out."""
        self._check(self.lib.wg_clear_error(self.h), "clear_error")

    def barrier_test(self, extra_arrivals: int):
        """wg_set_barrier_test: make the grid-barrier waits run out (failure-detection tests)."""
        self._check(self.lib.wg_set_barrier_test(self.h, int(extra_arrivals)), "set_barrier_test")

    # ---- water temperature (water_temp=True)
    def upload_longwave(self, day0: int, lw):
        """wg_upload_longwave: downward longwave [ndays, ncell] W/m2 into forcing slots day0.."""
        a = np.ascontiguousarray(lw, np.float32)
        assert a.ndim == 2 and a.shape[1] == self.region.ncell
        self._check(self.lib.wg_upload_longwave(self.h, int(day0), int(a.shape[0]), a.ctypes.data), "upload_longwave")

    def set_water_temp_inputs(self, gw_temp=None, river_length_check=None):
        """wg_set_water_temp_inputs: yearly groundwater temperature [ncell] and the river
        length as read (55 = no river), either may be None."""
        g = None if gw_temp is None else np.ascontiguousarray(gw_temp, np.float32)
        r = None if river_length_check is None else np.ascontiguousarray(river_length_check, np.float64)
        self._check(self.lib.wg_set_water_temp_inputs(self.h, None if g is None else g.ctypes.data,
                                                      None if r is None else r.ctypes.data), "set_water_temp_inputs")

    def water_temp(self):
        """(temperature [6, ncell], ice thickness [6, ncell]); rows: river, local lake,
        local wetland, global lake, reservoir, global wetland."""
        n = self.region.ncell
        t, i = np.empty((6, n)), np.empty((6, n))
        self._check(self.lib.wg_get_water_temp(self.h, t.ctypes.data, i.ctypes.data), "get_water_temp")
        return t, i

    def set_water_temp(self, temp=None, ice=None):
        t = None if temp is None else np.ascontiguousarray(temp, np.float64)
        i = None if ice is None else np.ascontiguousarray(ice, np.float64)
        self._check(self.lib.wg_set_water_temp(self.h, None if t is None else t.ctypes.data,
                                               None if i is None else i.ctypes.data), "set_water_temp")

    def river_temp(self, day0: int, ndays: int) -> np.ndarray:
        """River temperature of the stations' cells after each output day [ndays, nstation]."""
        out = np.empty((ndays, self.stations.size))
        self._check(self.lib.wg_get_river_temp(self.h, int(day0), int(ndays), out.ctypes.data), "get_river_temp")
        return out

    # ---- water use (water_use=True)
    def upload_water_use(self, fday0: int, ndays: int, doy0: int, nus, nug, irrig_withdrawal, irrig_consumptive):
        """wg_upload_water_use: one year's monthly net abstractions [12, ncell] (m3 per month)
        for forcing slots fday0 .. fday0+ndays-1, the first on day of year doy0."""
        arrs = [np.ascontiguousarray(a, np.float64) for a in (nus, nug, irrig_withdrawal, irrig_consumptive)]
        for a in arrs:
            if a.shape != (12, self.region.ncell):
                raise ValueError("water-use tables are [12, ncell]")
        self._check(self.lib.wg_upload_water_use(self.h, int(fday0), int(ndays), int(doy0),
                                                 *[a.ctypes.data for a in arrs]), "upload_water_use")

    def upload_water_use_run(self, fday0: int, doy0: int, ndays: int, use):
        """The tables of a whole run: use = (nus, nug, irrigation withdrawal, irrigation
        consumptive use), each [years, 12, ncell]; year k of the run (a new year at every
        day 1 after the first day) takes table k."""
        from .region import year_spans
        for d, m, doy, k in year_spans(doy0, ndays):
            self.upload_water_use(fday0 + d, m, doy, *(u[k] for u in use))

    def set_water_use_inputs(self, frac_return_gw_irrig):
        """wg_set_water_use_inputs: fraction of irrigation return flow into groundwater [ncell]."""
        a = np.ascontiguousarray(frac_return_gw_irrig, np.float64)
        self._check(self.lib.wg_set_water_use_inputs(self.h, a.ctypes.data), "set_water_use_inputs")

    def _wu_shape(self):
        k = WU_NSTATE
        return (k, self.region.ncell) if self.members == 1 else (k, self.region.ncell, self.members)

    def water_use(self) -> np.ndarray:
        """wg_get_water_use: the water-use state [13, ncell] (remaining, unsatisfied and
        actual use, a riparian cell's share of its outflow cell's unmet use);
        [13, ncell, members] for ensembles."""
        out = np.empty(self._wu_shape())
        self._check(self.lib.wg_get_water_use(self.h, out.ctypes.data), "get_water_use")
        return out

    def set_water_use(self, state):
        a = np.ascontiguousarray(state, np.float64)
        if a.shape != self._wu_shape():
            raise ValueError(f"water-use state is {self._wu_shape()}")
        self._check(self.lib.wg_set_water_use(self.h, a.ctypes.data), "set_water_use")

    def vertical_overlap(self, enable: bool | None = None) -> int:
        """Switch the vertical overlap on or off if given; return the extra warps per block (0: off)."""
        if enable is not None:
            self._check(self.lib.wg_set_vertical_overlap(self.h, int(bool(enable))), "set_vertical_overlap")
        return int(self.lib.wg_get_vertical_overlap(self.h))

    def autotune(self, doy0: int, fday0: int, ndays: int, t_begin: int, trial_steps: int) -> dict:
        """wg_autotune: pick threads per block and chunk steps on a trial window; state unchanged."""
        r = _TuneResult()
        self._check(self.lib.wg_autotune(self.h, int(doy0), int(fday0), int(ndays), int(t_begin), int(trial_steps),
                                         ctypes.byref(r)), "autotune")
        return {"threads": r.threads, "blocks": r.blocks, "chunk_steps": r.chunk_steps, "trials": r.trials,
                "ms_per_step": r.ms_per_step}

    def graph_capture(self, doy0: int, fday0: int, ndays: int, t_begin: int, t_end: int):
        self._check(self.lib.wg_graph_capture(self.h, int(doy0), int(fday0), int(ndays), int(t_begin), int(t_end)),
                    "graph_capture")

    def graph_launch(self):
        self._check(self.lib.wg_graph_launch(self.h), "graph_launch")

    def run(self, doy0: int, P, T, S, per_day: bool = False, chunk: int | None = None):
        """Convenience: upload forcing and simulate len(P) days from day-of-year doy0;
        returns station discharge [ndays, nstation]."""
        nd = P.shape[0]
        chunk = chunk or self.max_days
        qs = []
        done = 0
        doy = doy0
        while done < nd:
            k = min(chunk, nd - done, self.max_days)
            self.upload_forcing(0, P[done:done + k], T[done:done + k], S[done:done + k])
            if per_day:
                for d in range(k):
                    dd = (doy - 1 + d) % 365 + 1
                    self.step_vertical(dd, d)
                    self.step_routing(dd, d)
            else:
                self.run_days(doy, 0, k)
            qs.append(self.discharge(0, k))
            done += k
            doy = (doy - 1 + k) % 365 + 1
        return np.concatenate(qs) if qs else np.zeros((0, self.stations.size))
