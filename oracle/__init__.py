"""ctypes binding of the CPU oracle (test infrastructure only).

Loaded by tests/, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of bench.py -- never by the GPU library.  The oracle
restates the reference's calcNewDay/routing in C (wg_oracle.c); ``build()``
compiles it with ``make`` into ``oracle/_build``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libwg_oracle.so")
_lib = None

_STATIC_FIELDS = [
    ("ncell", ctypes.c_int32), ("nband", ctypes.c_int32), ("river_velo_opt", ctypes.c_int32),
    ("frac_routing", ctypes.c_int32), ("default_velocity", ctypes.c_double),
    ("lct_albedo", ctypes.c_void_p), ("lct_albedo_snow", ctypes.c_void_p), ("lct_ddf", ctypes.c_void_p),
    ("lct_lai_a", ctypes.c_void_p), ("lct_lai_b", ctypes.c_void_p), ("lct_initial_days", ctypes.c_void_p),
    ("area_km2", ctypes.c_void_p), ("lat_deg", ctypes.c_void_p), ("contfreq", ctypes.c_void_p),
    ("lct", ctypes.c_void_p), ("built_up", ctypes.c_void_p), ("smax", ctypes.c_void_p),
    ("lai_max", ctypes.c_void_p), ("gw_factor", ctypes.c_void_p), ("rg_max", ctypes.c_void_p),
    ("texture", ctypes.c_void_p), ("ldd", ctypes.c_void_p), ("aindex", ctypes.c_void_p),
    ("elev", ctypes.c_void_p), ("param", ctypes.c_void_p),
    ("loc_lake", ctypes.c_void_p), ("loc_wetl", ctypes.c_void_p), ("glo_wetl", ctypes.c_void_p),
    ("glo_lake", ctypes.c_void_p), ("glo_res", ctypes.c_void_p),
    ("lake_area", ctypes.c_void_p), ("res_area", ctypes.c_void_p), ("stor_cap", ctypes.c_void_p),
    ("mean_outflow", ctypes.c_void_p), ("mean_demand", ctypes.c_void_p), ("res_type", ctypes.c_void_p),
    ("start_month", ctypes.c_void_p),
    ("river_length", ctypes.c_void_p), ("river_slope", ctypes.c_void_p), ("roughness", ctypes.c_void_p),
    ("bankfull", ctypes.c_void_p), ("downstream", ctypes.c_void_p), ("rout_order", ctypes.c_void_p),
    ("statcorr_opt", ctypes.c_int32),
]

_STATE_ORDER = ["canopy", "soil", "snow", "snow_band", "lai_days", "lai_status", "lai_precsum",
                "gw", "river", "loclake", "locwetl", "glolake", "glowetl", "res",
                "rf_loclake", "rf_locwetl", "rf_glolake", "rf_glowetl", "rf_res", "k_release",
                "laf", "laf_prev", "fswb_next", "laf_started"]


class _Static(ctypes.Structure):
    _fields_ = _STATIC_FIELDS


class _State(ctypes.Structure):
    _fields_ = [(f, ctypes.c_void_p) for f in _STATE_ORDER]


class _WtIO(ctypes.Structure):
    _fields_ = [(f, ctypes.c_void_p) for f in ("longwave", "gw_temp", "inflow_cells", "river_length_check",
                                               "temp", "ice", "river_avail", "daily_temp")]


class _WuIO(ctypes.Structure):
    _fields_ = [(f, ctypes.c_void_p) for f in ("nus", "nug", "wdr", "cons", "row_of_day", "frgi", "state",
                                               "daily_actual")] + [("delayed", ctypes.c_int32)] + \
               [("nus_agg", ctypes.c_void_p), ("glwd_unit", ctypes.c_void_p)]


WU_NSTATE = 13
_DAYS_IN_MONTH = np.array([31, 28, 31, 30, 31, 30, 31, 31, 30, 31, 30, 31], np.float64)


def aggregate_nus(region, glwd_unit, nus_m3) -> np.ndarray:
    """dailyNUInit's aggregation over GLWD units (routing.cpp:926-965) of NUs
    [years, 12, ncell] m3 per month, month by month (wgo_aggregate_nus)."""
    nus = np.asarray(nus_m3, np.float64)
    unit = np.ascontiguousarray(glwd_unit, np.int32)
    lake = np.ascontiguousarray(region.lake_area, np.float64)
    res = np.ascontiguousarray(region.res_area, np.float64)
    out = np.empty_like(nus)
    flat_in, flat_out = nus.reshape(-1, nus.shape[-1]), out.reshape(-1, nus.shape[-1])
    for k in range(flat_in.shape[0]):
        src = np.ascontiguousarray(flat_in[k])
        dst = np.empty_like(src)
        if lib().wgo_aggregate_nus(region.ncell, _ptr(lake), _ptr(res), _ptr(unit), _ptr(src), _ptr(dst)):
            raise ValueError("GLWD units: every global lake or reservoir outflow cell needs a unit > 0, "
                             "one outflow cell per unit")
        flat_out[k] = dst
    return out


def daily_use(m3_per_month) -> np.ndarray:
    """dailyNUInit's conversion (routing.cpp:966-975): m3 per month [..., 12, ncell]
    -> km3 per day, the multipliers M_NETABSSW/M_NETABSGW being 1."""
    v = np.asarray(m3_per_month, np.float64)
    return v / (1000000000. * _DAYS_IN_MONTH[:, None])


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB)
        _lib.wgo_init_state.argtypes = [ctypes.POINTER(_Static), ctypes.POINTER(_State)]
        _lib.wgo_run.argtypes = [ctypes.POINTER(_Static), ctypes.POINTER(_State), ctypes.c_int, ctypes.c_int,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.c_int]
        _lib.wgo_last_timing.argtypes = [ctypes.c_void_p]
        _lib.wgo_bottom_width.argtypes = [ctypes.c_double]
        _lib.wgo_aggregate_nus.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 5
        _lib.wgo_aggregate_nus.restype = ctypes.c_int
        _lib.wgo_bottom_width.restype = ctypes.c_double
        _lib.wgo_wtemp_batch.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        _lib.wgo_wt_init.argtypes = [ctypes.c_int, ctypes.POINTER(_WtIO)]
        _lib.wgo_run_wt.argtypes = [ctypes.POINTER(_Static), ctypes.POINTER(_State), ctypes.c_int, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_WtIO)]
        _lib.wgo_run_wu.argtypes = [ctypes.POINTER(_Static), ctypes.POINTER(_State), ctypes.c_int, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_WuIO)]
        _lib.wgo_run_wt_wu.argtypes = [ctypes.POINTER(_Static), ctypes.POINTER(_State), ctypes.c_int, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_WtIO), ctypes.POINTER(_WuIO)]
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


WT_NIN = 73   # doubles per water-temperature record (wgo_wt_in)


def wtemp(records: np.ndarray) -> np.ndarray:
    """wgo_wtemp on each row of records [n, 73]; returns [n, 12] (temperatures, ice)."""
    rec = np.ascontiguousarray(records, np.float64)
    assert rec.ndim == 2 and rec.shape[1] == WT_NIN
    out = np.empty((rec.shape[0], 12))
    lib().wgo_wtemp_batch(_ptr(rec), int(rec.shape[0]), _ptr(out))
    return out


class Oracle:
    """One region simulated by the CPU restatement; state arrays live in ``self.state``."""

    def __init__(self, region):
        from watergap2_gb300.region import empty_state
        self.region = region
        self._keep = []
        st = _Static()
        st.ncell, st.nband = region.ncell, region.nband
        st.river_velo_opt, st.default_velocity = region.river_velo_opt, region.default_velocity
        st.frac_routing = int(getattr(region, "frac_routing", 0))
        for name, ctype in _STATIC_FIELDS[5:-1]:
            a = region.arrays[name]
            self._keep.append(a)
            setattr(st, name, a.ctypes.data)
        st.statcorr_opt = int(getattr(region, "statcorr_opt", 0))
        self._static = st
        self.state = empty_state(region.ncell, region.nband)
        self._cstate = _State()
        for f in _STATE_ORDER:
            setattr(self._cstate, f, self.state[f].ctypes.data)
        rc = lib().wgo_init_state(ctypes.byref(self._static), ctypes.byref(self._cstate))
        if rc:
            raise RuntimeError(f"wgo_init_state failed: {rc}")

    def init_water_temp(self, gw_temp, river_length_check=None):
        """Switch on the water temperature: the reference's start values (15 degC,
        no ice); gw_temp [ncell] the yearly groundwater temperature; the river
        length check defaults to the region's river length as read."""
        from watergap2_gb300.region import inflow_cells
        n = self.region.ncell
        self.wt = {"temp": np.zeros((6, n)), "ice": np.zeros((6, n)), "river_avail": np.zeros(n)}
        self._wt_static = {
            "gw_temp": np.ascontiguousarray(gw_temp, np.float32),
            "inflow_cells": np.ascontiguousarray(inflow_cells(self.region), np.int32),
            "river_length_check": np.ascontiguousarray(
                self.region.extras["river_length_file"] if river_length_check is None else river_length_check,
                np.float64),
        }
        io = self._wt_io(None, None)
        lib().wgo_wt_init(n, ctypes.byref(io))

    def _wt_io(self, lw, daily):
        io = _WtIO()
        io.longwave = _ptr(lw) if lw is not None else None
        for k, v in self._wt_static.items():
            setattr(io, k, _ptr(v))
        for k, v in self.wt.items():
            setattr(io, k, _ptr(v))
        io.daily_temp = _ptr(daily) if daily is not None else None
        return io

    def run_wt(self, doy0, P, T, S, LW, discharge=False, daily_temp=False, nthreads=1):
        """run() with the water temperature; returns (discharge, daily out[0] of every cell)."""
        P, T, S, LW = (np.ascontiguousarray(x, np.float32) for x in (P, T, S, LW))
        nd = P.shape[0]
        q = np.zeros((nd, self.region.ncell)) if discharge else None
        dt = np.zeros((nd, self.region.ncell)) if daily_temp else None
        io = self._wt_io(LW, dt)
        rc = lib().wgo_run_wt(ctypes.byref(self._static), ctypes.byref(self._cstate), int(doy0), nd,
                              _ptr(P), _ptr(T), _ptr(S), _ptr(q) if q is not None else None, None,
                              int(nthreads), ctypes.byref(io))
        if rc:
            raise RuntimeError(f"wgo_run_wt failed: {rc}")
        return q, dt

    def init_water_use(self, frac_return_gw_irrig, delayed=False, glwd_unit=None):
        """Switch on water use: its state starts at zero (routing.cpp:790-848);
        frac_return_gw_irrig [ncell] is G_fractreturngw_irrig; delayed: unmet
        demand carried to the next day (options.delayedUseSatisfaction);
        glwd_unit [ncell] (G_glwdUnit, 0 none): aggrNUsGloLakResOpt = 1, the
        riparian cells' NUs met by their global lake's or reservoir's outflow cell."""
        self.wu = np.zeros((WU_NSTATE, self.region.ncell))
        self._wu_delayed = int(bool(delayed))
        self._wu_frgi = np.ascontiguousarray(frac_return_gw_irrig, np.float64)
        self._wu_unit = None if glwd_unit is None else np.ascontiguousarray(glwd_unit, np.int32)

    def _wu_tables(self, doy0, nd, use):
        """The daily tables of run_wu (and the GLWD-aggregated NUs where
        init_water_use had units): ([nus, nug, wdr, cons], rows, nus_agg or None)."""
        from watergap2_gb300.region import use_rows
        n = self.region.ncell
        tabs = [np.ascontiguousarray(daily_use(u).reshape(-1, n)) for u in use]
        rows = np.ascontiguousarray(use_rows(doy0, nd), np.int32)
        if rows.max() >= tabs[0].shape[0]:
            raise ValueError("water use covers fewer years than the run")
        agg = None
        if self._wu_unit is not None:
            agg = np.ascontiguousarray(daily_use(aggregate_nus(self.region, self._wu_unit, use[0])).reshape(-1, n))
        return tabs, rows, agg

    def _wu_io(self, tabs, rows, agg, da=None):
        io = _WuIO()
        io.nus, io.nug, io.wdr, io.cons = (_ptr(t) for t in tabs)
        io.row_of_day, io.frgi, io.state = _ptr(rows), _ptr(self._wu_frgi), _ptr(self.wu)
        io.daily_actual = _ptr(da) if da is not None else None
        io.delayed = self._wu_delayed
        io.nus_agg = _ptr(agg) if agg is not None else None
        io.glwd_unit = _ptr(self._wu_unit) if agg is not None else None
        return io

    def run_wt_wu(self, doy0, P, T, S, LW, use, discharge=False, daily_temp=False, nthreads=1):
        """run() with the water temperature (init_water_temp) and water use
        (init_water_use); returns (discharge, daily out[0] of every cell)."""
        P, T, S, LW = (np.ascontiguousarray(x, np.float32) for x in (P, T, S, LW))
        nd, n = P.shape[0], self.region.ncell
        tabs, rows, agg = self._wu_tables(doy0, nd, use)
        q = np.zeros((nd, n)) if discharge else None
        dt = np.zeros((nd, n)) if daily_temp else None
        wt = self._wt_io(LW, dt)
        io = self._wu_io(tabs, rows, agg)
        rc = lib().wgo_run_wt_wu(ctypes.byref(self._static), ctypes.byref(self._cstate), int(doy0), nd,
                                 _ptr(P), _ptr(T), _ptr(S), _ptr(q) if q is not None else None, None,
                                 int(nthreads), ctypes.byref(wt), ctypes.byref(io))
        if rc:
            raise RuntimeError(f"wgo_run_wt_wu failed: {rc}")
        return q, dt

    def run_wu(self, doy0, P, T, S, use, discharge=False, balance=False, daily_actual=False, nthreads=1):
        """run() with water use.  use = (nus, nug, irrigation withdrawal, irrigation
        consumptive use), each [years, 12, ncell] m3 per month; the first day is in
        year 0 and every day of year 1 of the day-of-year count starts the next
        year, as the reference's driver reads the yearly files.  Returns
        (discharge, balance, daily actual use [ndays, ncell] km3)."""
        P, T, S = (np.ascontiguousarray(x, np.float32) for x in (P, T, S))
        nd, n = P.shape[0], self.region.ncell
        tabs, rows, agg = self._wu_tables(doy0, nd, use)
        q = np.zeros((nd, n)) if discharge else None
        b = np.zeros((nd, 6)) if balance else None
        da = np.zeros((nd, n)) if daily_actual else None
        io = self._wu_io(tabs, rows, agg, da)
        rc = lib().wgo_run_wu(ctypes.byref(self._static), ctypes.byref(self._cstate), int(doy0), nd,
                              _ptr(P), _ptr(T), _ptr(S), _ptr(q) if q is not None else None,
                              _ptr(b) if b is not None else None, int(nthreads), ctypes.byref(io))
        if rc:
            raise RuntimeError(f"wgo_run_wu failed: {rc}")
        return q, b, da

    def run(self, doy0, P, T, S, discharge=False, balance=False, nthreads=1):
        P, T, S = (np.ascontiguousarray(x, np.float32) for x in (P, T, S))
        nd = P.shape[0]
        assert P.shape == (nd, self.region.ncell)
        q = np.zeros((nd, self.region.ncell)) if discharge else None
        b = np.zeros((nd, 6)) if balance else None
        rc = lib().wgo_run(ctypes.byref(self._static), ctypes.byref(self._cstate), int(doy0), nd,
                           _ptr(P), _ptr(T), _ptr(S), _ptr(q) if q is not None else None,
                           _ptr(b) if b is not None else None, int(nthreads))
        if rc:
            raise RuntimeError(f"wgo_run failed: {rc}")
        return q, b

    @staticmethod
    def last_timing() -> dict:
        """Wall time of the vertical and the routing pass of the last run."""
        out = np.zeros(2)
        lib().wgo_last_timing(_ptr(out))
        return {"vertical_s": float(out[0]), "routing_s": float(out[1])}
