"""Seeded synthetic regions and forcing for the daily step.

No public dataset is involved: the inputs of each workload are generated here
from fixed seeds with the sizes and value distributions of the workloads the
GB300 library is measured on:

* ``region_64x64``  -- 64 x 64 block of 0.5-degree cells, all land, D8 drainage
  from a fractal elevation field with pits filled and a single outlet; no
  lakes, wetlands or reservoirs.
* ``region_global`` -- 360 x 720 0.5-degree grid with 67,420 land cells from a
  seeded land mask, D8 drainage with about 6,000 outlets plus a few inland
  sinks; local lakes in 3 % of the cells, wetlands in 2 %, 300 global lakes and
  1,200 reservoirs (capacity lognormal(ln 50 hm3, 1.5)), Manning n ~ U(0.02, 0.1).
* ``forcing``       -- daily precipitation (0 with probability 0.6, else
  Gamma(k=0.8, theta=8 mm)), temperature 10 + 12 sin(2 pi d/365) + N(0, 3) C
  (shifted and mirrored with latitude on the global grid) and shortwave
  50-300 W/m2 with the seasons.

Every quantity the reference reads from a float UNF grid or a ``short``/``char``
grid is rounded to that type here, so that the reference and this library see
identical inputs.
"""
from __future__ import annotations

import heapq
import math

import os

import numpy as np

from .region import NLCT, NPARAM, PARAM, Region

EARTH_R_KM = 6371.0
# keypad codes of the reference's LDD (source/rout_prepare.cpp:619-670):
# code -> (d_row, d_col) with rows counted from the north (row index grows southwards)
LDD_STEP = {1: (1, -1), 2: (1, 0), 3: (1, 1), 4: (0, -1), 6: (0, 1), 7: (-1, -1), 8: (-1, 0), 9: (-1, 1)}
STEP_LDD = {v: k for k, v in LDD_STEP.items()}


def cell_area_km2(row: np.ndarray, res: float = 0.5) -> np.ndarray:
    """Area of a res-degree cell in grid row ``row`` (1-based, north to south), float32."""
    lat_n = np.radians(90.0 - (row - 1) * res)
    lat_s = np.radians(90.0 - row * res)
    a = EARTH_R_KM ** 2 * np.radians(res) * (np.sin(lat_n) - np.sin(lat_s))
    return np.abs(a).astype(np.float32)


def row_latitude(row: np.ndarray, res: float = 0.5) -> np.ndarray:
    """Cell-centre latitude; for 0.5 degrees the reference's -(G_row/2 - 90.25)
    (source/daily.cpp:2423), which only exists for that grid."""
    if res == 0.5:
        return -(row.astype(np.float64) / 2.0 - 90.25)
    return 90.0 - (row.astype(np.float64) - 0.5) * res


def fractal_field(shape, beta: float, rng: np.random.Generator) -> np.ndarray:
    """Spectral-synthesis fractal surface with power spectrum ~ k^-beta, scaled to [0, 1]."""
    ny, nx = shape
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.rfftfreq(nx)[None, :]
    k = np.sqrt(kx * kx + ky * ky)
    k[0, 0] = 1.0
    amp = k ** (-beta / 2.0)
    amp[0, 0] = 0.0
    phase = rng.uniform(0, 2 * np.pi, size=amp.shape)
    spec = amp * (np.cos(phase) + 1j * np.sin(phase))
    f = np.fft.irfft2(spec, s=shape)
    f -= f.min()
    f /= max(f.max(), 1e-30)
    return f


def _neighbours(r, c, ny, nx, wrap):
    for dr in (-1, 0, 1):
        for dc in (-1, 0, 1):
            if dr == 0 and dc == 0:
                continue
            rr, cc = r + dr, c + dc
            if rr < 0 or rr >= ny:
                continue
            if cc < 0 or cc >= nx:
                if not wrap:
                    continue
                cc %= nx
            yield rr, cc, dr, dc


def _synth_lib():
    import ctypes
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libwg_synth.so")
    if not os.path.exists(path):
        return None
    lib = ctypes.CDLL(path)
    lib.wg_synth_flood_d8.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    lib.wg_synth_flood_d8.restype = ctypes.c_int
    return lib


def flood_and_d8(dem: np.ndarray, land: np.ndarray, seeds: np.ndarray, wrap: bool, native: bool | None = None):
    """Priority-flood pit filling from the seed cells, then D8 steepest descent on
    the filled surface.  Returns ldd codes (5 at seeds, 1-9 elsewhere, 0 off-land).
    Uses the compiled helper (libwg_synth.so, same algorithm) when present."""
    ny, nx = dem.shape
    lib = _synth_lib() if native is not False else None
    if lib is not None:
        d = np.ascontiguousarray(dem, np.float64)
        la = np.ascontiguousarray(land, np.uint8)
        se = np.ascontiguousarray(seeds, np.uint8).copy()
        ldd = np.zeros((ny, nx), np.int8)
        rc = lib.wg_synth_flood_d8(ny, nx, d.ctypes.data, la.ctypes.data, se.ctypes.data, int(bool(wrap)),
                                   ldd.ctypes.data)
        if rc:
            raise RuntimeError("cell without a downhill neighbour after pit filling")
        return ldd, None
    eps = 1e-6
    filled = np.full(dem.shape, np.inf)
    done = np.zeros(dem.shape, bool)
    heap = []
    seeds = seeds.copy()
    for r, c in zip(*np.nonzero(seeds)):
        filled[r, c] = dem[r, c]
        heapq.heappush(heap, (dem[r, c], int(r), int(c)))
        done[r, c] = True
    while True:
        while heap:
            z, r, c = heapq.heappop(heap)
            for rr, cc, _, _ in _neighbours(r, c, ny, nx, wrap):
                if not land[rr, cc] or done[rr, cc]:
                    continue
                done[rr, cc] = True
                zz = max(dem[rr, cc], z + eps)
                filled[rr, cc] = zz
                heapq.heappush(heap, (zz, rr, cc))
        left = land & ~done
        if not left.any():
            break
        # a land component no seed reaches (an island): its lowest cell becomes its outlet
        lr, lc = np.nonzero(left)
        k = int(np.argmin(dem[lr, lc]))
        r, c = int(lr[k]), int(lc[k])
        seeds[r, c] = True
        done[r, c] = True
        filled[r, c] = dem[r, c]
        heapq.heappush(heap, (dem[r, c], r, c))
    ldd = np.zeros(dem.shape, np.int8)
    sq2 = math.sqrt(2.0)
    for r, c in zip(*np.nonzero(land)):
        if seeds[r, c]:
            ldd[r, c] = 5
            continue
        best, code = 0.0, 0
        for rr, cc, dr, dc in _neighbours(r, c, ny, nx, wrap):
            if not land[rr, cc]:
                continue
            drop = (filled[r, c] - filled[rr, cc]) / (sq2 if dr and dc else 1.0)
            if drop > best:
                best, code = drop, STEP_LDD[(dr, dc)]
        if code == 0:
            raise RuntimeError("cell without a downhill neighbour after pit filling")
        ldd[r, c] = code
    return ldd, filled


def routing_levels(downstream: np.ndarray) -> np.ndarray:
    """Pass number of the reference's Kahn routing order (source/rout_prepare.cpp:834-886):
    cells without inflow get 1, every other cell 1 + the largest pass of its inflows."""
    n = downstream.shape[0]
    indeg = np.bincount(downstream[downstream >= 0], minlength=n).astype(np.int64)
    level = np.zeros(n, np.int64)
    frontier = np.nonzero(indeg == 0)[0]
    p = 1
    seen = 0
    while frontier.size:
        level[frontier] = p
        seen += frontier.size
        d = downstream[frontier]
        d = d[d >= 0]
        np.subtract.at(indeg, d, 1)
        cand = np.unique(d)
        frontier = cand[indeg[cand] == 0]
        p += 1
    if seen != n:
        raise ValueError("drainage network has a cycle")
    return level


def rout_order_from(downstream: np.ndarray) -> np.ndarray:
    """Cells in the reference's routing order: by pass, ties by cell index."""
    return np.argsort(routing_levels(downstream), kind="stable").astype(np.int32)


def _lct_tables(rng: np.random.Generator):
    albedo = np.round(rng.uniform(0.10, 0.25, NLCT), 3)
    albedo_snow = np.round(rng.uniform(0.40, 0.75, NLCT), 3)
    ddf = np.round(rng.uniform(1.5, 6.0, NLCT), 2)
    lai = np.round(rng.uniform(0.5, 6.0, NLCT), 2).astype(np.float32)
    fdp = np.round(rng.uniform(0.0, 1.0, NLCT), 2).astype(np.float32)
    rfep = np.round(rng.uniform(0.5, 1.0, NLCT), 2).astype(np.float32)
    # laiClass::init (source/lai.cpp:86-90): a = 0.1*fdp (double -> float), b = (1-fdp)*rfep (float)
    lai_a = (0.1 * fdp.astype(np.float64)).astype(np.float32)
    lai_b = ((np.float32(1.0) - fdp) * rfep).astype(np.float32)
    initial_days = rng.integers(5, 30, NLCT).astype(np.int16)
    kc_min = np.round(rng.uniform(0.3, 0.6, NLCT), 2)
    kc_max = np.round(rng.uniform(0.9, 1.2, NLCT), 2)
    emissivity = np.round(rng.uniform(0.95, 0.99, NLCT), 3)
    rooting = np.round(rng.uniform(0.5, 4.0, NLCT), 2)
    return dict(albedo=albedo, albedo_snow=albedo_snow, ddf=ddf, lai=lai, fdp=fdp, rfep=rfep,
                lai_a=lai_a, lai_b=lai_b, initial_days=initial_days, kc_min=kc_min, kc_max=kc_max,
                emissivity=emissivity, rooting=rooting)


def _upstream_cells(downstream: np.ndarray, order: np.ndarray) -> np.ndarray:
    """Number of cells draining through each cell (itself included)."""
    acc = np.ones(downstream.shape[0], np.int64)
    for n in order:
        d = downstream[n]
        if d >= 0:
            acc[d] += acc[n]
    return acc


def _build_region(name, rows, cols, gr, gc, ldd_grid, index_grid, dem_m, coastal, rng, nband, swb, river_velo_opt,
                  wrap=False, res=0.5):
    """rows/cols: global 1-based 0.5-degree position; gr/gc: 0-based position in ldd_grid."""
    ncell = rows.shape[0]
    tabs = _lct_tables(np.random.default_rng(7))
    # downstream cell from the ldd codes
    downstream = np.full(ncell, -1, np.int32)
    ny, nx = index_grid.shape
    ldd = ldd_grid[gr, gc].astype(np.int8)
    for i in range(ncell):
        code = int(ldd[i])
        if code in LDD_STEP:
            dr, dc = LDD_STEP[code]
            rr, cc = gr[i] + dr, gc[i] + dc
            if wrap:
                cc %= nx
            downstream[i] = index_grid[rr, cc]
            assert downstream[i] >= 0
    order = rout_order_from(downstream)
    acc = _upstream_cells(downstream, order)

    area = cell_area_km2(rows, res).astype(np.float64)
    lat = row_latitude(rows, res)
    contfreq = np.where(coastal, np.round(rng.uniform(40.0, 100.0, ncell), 1), 100.0).astype(np.float32)
    contfreq = contfreq.astype(np.float64)
    lct = rng.integers(1, NLCT + 1, ncell).astype(np.uint8)
    built_up = np.where(rng.uniform(size=ncell) < 0.1, rng.uniform(0.0, 0.05, ncell), 0.0).astype(np.float32)
    smax = rng.uniform(50.0, 500.0, ncell).astype(np.float32)
    lai_max = rng.uniform(0.5, 6.0, ncell).astype(np.float32)
    gw_factor = rng.uniform(0.1, 0.9, ncell).astype(np.float32)
    rg_max = rng.integers(100, 700, ncell).astype(np.int16)
    texture = rng.integers(10, 31, ncell).astype(np.int8)
    aindex = (rng.uniform(size=ncell) < 0.3).astype(np.int16)
    mean_elev = np.round(dem_m).astype(np.int32)
    offs = rng.uniform(0.0, 1500.0, (ncell, nband)) * rng.choice([-1.0, 1.0], (ncell, nband))
    offs = np.sort(np.round(offs), axis=1)
    bands = np.clip(mean_elev[:, None] + offs, -400, 8800).astype(np.int16)
    elev = np.concatenate([mean_elev[:, None].astype(np.int16), bands], axis=1)

    par = np.zeros((NPARAM, ncell))
    par[PARAM["P_GAMRUN_C"]] = rng.uniform(0.1, 5.0, ncell)
    par[PARAM["P_CFA"]] = 1.0
    par[PARAM["P_CFS"]] = 1.0
    par[PARAM["M_ROOT_D"]] = 1.0
    par[PARAM["M_RIVRGH_C"]] = 1.0
    par[PARAM["P_LAK_D"]] = 5.0
    par[PARAM["P_WET_D"]] = 2.0
    par[PARAM["P_SWOUTF_C"]] = 0.01
    par[PARAM["M_EVAREDEX"]] = 1.0
    par[PARAM["M_NETRAD"]] = 1.0
    par[PARAM["P_PTC_HUM"]] = 1.26
    par[PARAM["P_PTC_ARI"]] = 1.74
    par[PARAM["P_PET_MXDY"]] = 15.0
    par[PARAM["P_MCWH"]] = 0.3
    par[PARAM["M_LAI"]] = 1.0
    par[PARAM["P_T_SNOWFZ"]] = 0.0
    par[PARAM["P_T_SNOWMT"]] = 0.0
    par[PARAM["M_DEGDAY_F"]] = 1.0
    par[PARAM["P_T_GRADNT"]] = 0.006
    par[PARAM["M_GW_F"]] = 1.0
    par[PARAM["M_RG_MAX"]] = 1.0
    par[PARAM["P_PCRITGWA"]] = 12.5
    par[PARAM["P_GWOUTF_C"]] = 0.01
    par[PARAM["M_NETABSSW"]] = 1.0
    par[PARAM["M_NETABSGW"]] = 1.0
    par[PARAM["M_PREC"]] = 1.0

    z = np.zeros(ncell)
    loc_lake, loc_wetl, glo_wetl, glo_lake, glo_res = z.copy(), z.copy(), z.copy(), z.copy(), z.copy()
    lake_area, res_area, stor_cap, mean_outflow, mean_demand = z.copy(), z.copy(), z.copy(), z.copy(), z.copy()
    mean_outflow_file = z.copy()
    res_type = np.full(ncell, 2, np.int8)
    start_month = np.ones(ncell, np.int8)
    if swb is not None:
        n_loclake, n_wetl, n_glolake, n_res = swb
        perm = rng.permutation(ncell)
        i0 = 0
        sel = perm[i0:i0 + n_loclake]; i0 += n_loclake
        loc_lake[sel] = np.round(rng.uniform(1.0, 30.0, sel.size), 2).astype(np.float32)
        sel = perm[i0:i0 + n_wetl]; i0 += n_wetl
        half = sel.size // 2
        loc_wetl[sel[:half]] = np.round(rng.uniform(1.0, 30.0, half), 2).astype(np.float32)
        glo_wetl[sel[half:]] = np.round(rng.uniform(1.0, 30.0, sel.size - half), 2).astype(np.float32)
        # global lakes and reservoirs sit in outflow cells with some upstream area
        cand = perm[i0:]
        cand = cand[acc[cand] >= 3]
        sel = cand[:n_glolake]
        frac = rng.uniform(5.0, 40.0, sel.size)
        glo_lake[sel] = np.round(frac, 2).astype(np.float32)
        lake_area[sel] = (glo_lake[sel] / 100.0 * area[sel]).astype(np.float32)
        sel = cand[n_glolake:n_glolake + n_res]
        cap_hm3 = np.exp(rng.normal(math.log(50.0), 1.5, sel.size))
        stor_cap[sel] = (cap_hm3 / 1000.0).astype(np.float32)
        ra = np.minimum(stor_cap[sel] / 0.01, 0.25 * area[sel] * contfreq[sel] / 100.0)
        res_area[sel] = np.maximum(ra, 0.5).astype(np.float32)
        glo_res[sel] = (res_area[sel] / area[sel] * 100.0).astype(np.float32)
        # long-term mean outflow, km3/month in the file (routing.cpp:455-461): 0.4 mm/d of upstream area
        up_km2 = acc[sel] * area[sel]
        km3_month = (up_km2 * 0.4e-6 * 30.4).astype(np.float32).astype(np.float64)
        mean_outflow_file[sel] = km3_month
        mean_outflow[sel] = km3_month * 12. * 1000000000. / 31536000.
        res_type[sel] = rng.integers(1, 3, sel.size).astype(np.int8)
        start_month[sel] = rng.integers(1, 13, sel.size).astype(np.int8)
        # keep the land fraction positive
        tot = loc_lake + loc_wetl + glo_wetl + glo_lake + glo_res
        over = tot > 0.8 * contfreq
        scale = np.where(over, 0.8 * contfreq / np.maximum(tot, 1e-9), 1.0)
        for a in (loc_lake, loc_wetl, glo_wetl, glo_lake, glo_res):
            a *= scale
            a[:] = a.astype(np.float32)
        lake_area[:] = np.where(glo_lake > 0, (glo_lake / 100.0 * area).astype(np.float32), 0.0)
        res_area[:] = np.where(glo_res > 0, np.maximum(res_area, 0.0), 0.0)

    raw_len = (rng.uniform(30.0, 80.0, ncell) * (res / 0.5)).astype(np.float32).astype(np.float64)
    river_length = raw_len * (contfreq / 100.)          # routing.cpp:480-482
    river_slope = np.exp(rng.uniform(math.log(1e-5), math.log(1e-2), ncell)).astype(np.float32).astype(np.float64)
    rough_hi = 0.1 if swb is not None else 0.05
    roughness = rng.uniform(0.02, rough_hi, ncell).astype(np.float32).astype(np.float64)
    bankfull = (0.02 * (acc * area) ** 0.8).astype(np.float32).astype(np.float64)

    arrays = dict(
        lct_albedo=tabs["albedo"], lct_albedo_snow=tabs["albedo_snow"], lct_ddf=tabs["ddf"],
        lct_lai_a=tabs["lai_a"], lct_lai_b=tabs["lai_b"], lct_initial_days=tabs["initial_days"],
        area_km2=area, lat_deg=lat, contfreq=contfreq, lct=lct, built_up=built_up, smax=smax,
        lai_max=lai_max, gw_factor=gw_factor, rg_max=rg_max, texture=texture, ldd=ldd,
        aindex=aindex, elev=elev.reshape(-1), param=par.reshape(-1),
        loc_lake=loc_lake, loc_wetl=loc_wetl, glo_wetl=glo_wetl, glo_lake=glo_lake, glo_res=glo_res,
        lake_area=lake_area, res_area=res_area, stor_cap=stor_cap, mean_outflow=mean_outflow,
        mean_demand=mean_demand, res_type=res_type, start_month=start_month,
        river_length=river_length, river_slope=river_slope, roughness=roughness, bankfull=bankfull,
        downstream=downstream, rout_order=order,
    )
    reg = Region(ncell=ncell, nband=nband, arrays=arrays, river_velo_opt=river_velo_opt,
                 row=rows.astype(np.int16), col=cols.astype(np.int16), name=name)
    reg.lct_tables = tabs
    # values as they appear in the reference's input files (before routing.init derives from them)
    reg.extras = dict(mean_outflow_km3_month=mean_outflow_file, river_length_file=raw_len)
    return reg


def region_64x64(seed: int = 1, nband: int = 5, row0: int = 60, col0: int = 300, size: int = 64) -> Region:
    """size x size (default 64 x 64) all-land 0.5-degree block, single outlet, no water bodies."""
    rng = np.random.default_rng(seed)
    ny = nx = size
    dem = fractal_field((ny, nx), 3.0, rng) * 2500.0
    # tilt towards the south-east corner so that the outlet is there
    yy, xx = np.mgrid[0:ny, 0:nx]
    dem = dem + 400.0 * (2.0 - yy / ny - xx / nx)
    land = np.ones((ny, nx), bool)
    seeds = np.zeros((ny, nx), bool)
    edge = np.zeros((ny, nx), bool)
    edge[0, :] = edge[-1, :] = edge[:, 0] = edge[:, -1] = True
    er, ec = np.nonzero(edge)
    k = np.argmin(dem[er, ec])
    seeds[er[k], ec[k]] = True
    ldd, filled = flood_and_d8(dem, land, seeds, wrap=False)
    rr, cc = np.nonzero(land)
    index = -np.ones((ny, nx), np.int64)
    index[rr, cc] = np.arange(rr.size)
    rows = (rr + row0).astype(np.int64)
    cols = (cc + col0).astype(np.int64)
    rng2 = np.random.default_rng(seed + 2)   # parameters: seed 3 in the default set
    coastal = np.zeros(rr.size, bool)
    reg = _build_region(f"region_{size}x{size}", rows, cols, rr, cc, ldd, index, dem[rr, cc], coastal, rng2, nband,
                        None, 1)
    return reg


def region_global(seed: int = 11, nband: int = 5, nland: int = 67420, n_outlets: int = 6000,
                  n_sinks: int = 60, swb=(2023, 1348, 300, 1200), river_velo_opt: int = 1,
                  shape=(360, 720), name: str = "region_global", block_at=None) -> Region:
    """Global 0.5-degree grid with a seeded land mask (default 67,420 land cells).
    With another shape the grid spacing is 180/ny degrees, unless block_at =
    (row0, col0) places the shape as a block of the 0.5-degree grid at that
    0-based offset (no wrap in longitude): the geometry the reference's own
    code reads."""
    rng = np.random.default_rng(seed)
    ny, nx = shape
    mask_f = fractal_field((ny, nx), 3.2, rng)
    lat_rows = np.arange(ny)
    allowed = (lat_rows >= int(ny * 12 / 360)) & (lat_rows < int(ny * 290 / 360))
    score = np.where(allowed[:, None], mask_f, -1.0)
    thr = np.sort(score.ravel())[-nland]
    land = score >= thr
    # exact count
    idx = np.flatnonzero(land)
    if idx.size > nland:
        land.ravel()[idx[np.argsort(score.ravel()[idx])[: idx.size - nland]]] = False
    dem = fractal_field((ny, nx), 3.0, rng) * 3000.0 + 600.0 * mask_f
    # coastal land cells
    ocean = ~land
    coastal = np.zeros_like(land)
    for dr in (-1, 0, 1):
        for dc in (-1, 0, 1):
            if dr or dc:
                sh = np.roll(np.roll(ocean, dr, axis=0), dc, axis=1)
                if dr == 1:
                    sh[0, :] = True
                if dr == -1:
                    sh[-1, :] = True
                coastal |= sh
    coastal &= land
    cr, cc_ = np.nonzero(coastal)
    pick = np.argsort(dem[cr, cc_])[:n_outlets]
    seeds = np.zeros_like(land)
    seeds[cr[pick], cc_[pick]] = True
    # a few inland sinks at interior local minima
    interior = land & ~coastal
    ir, ic = np.nonzero(interior)
    sel = rng.choice(ir.size, size=min(n_sinks, ir.size), replace=False)
    sinks = np.zeros_like(land)
    sinks[ir[sel], ic[sel]] = True
    wrap = block_at is None
    ldd, _ = flood_and_d8(dem, land, seeds | sinks, wrap=wrap)
    ldd[sinks] = -1
    rr, cc = np.nonzero(land)
    index = -np.ones((ny, nx), np.int64)
    index[rr, cc] = np.arange(rr.size)
    r0, c0 = block_at if block_at is not None else (0, 0)
    reg = _build_region(name, (rr + 1 + r0).astype(np.int64), (cc + 1 + c0).astype(np.int64), rr, cc, ldd, index,
                        dem[rr, cc], coastal[rr, cc], np.random.default_rng(seed + 2), nband, swb,
                        river_velo_opt, wrap=wrap, res=0.5 if block_at is not None else 180.0 / ny)
    return reg


def region_5min(seed: int = 41, nband: int = 5, nland: int = 2_200_000, shape=(2160, 4320)) -> Region:
    """Fine global grid: 2160 x 4320 cells of 5 arc-minutes, ~2.2 M land cells, the
    global generators at 9x the water-body counts.  The reference cannot run it
    (its geometry is fixed to 0.5 degrees, def.h:10, geo.h:25)."""
    k = 9
    return region_global(seed=seed, nband=nband, nland=nland, n_outlets=6000 * k, n_sinks=60 * k,
                         swb=(int(0.03 * nland), int(0.02 * nland), 300 * k, 1200 * k), shape=shape,
                         name="region_5min")


def region_small_swb(seed: int = 21, nband: int = 5, ny: int = 24, nx: int = 48,
                     river_velo_opt: int = 1, block_at=None) -> Region:
    """Small grid with every water-body type, inland sinks and coastal cells (parity
    tests); block_at = (row0, col0) puts it on the 0.5-degree grid (see region_global)."""
    nland = int(ny * nx * 0.55)
    return region_global(seed=seed, nband=nband, nland=nland, n_outlets=max(8, nland // 12), n_sinks=4,
                         swb=(max(4, nland // 20), max(4, nland // 20), max(3, nland // 60), max(4, nland // 40)),
                         river_velo_opt=river_velo_opt, shape=(ny, nx), block_at=block_at)


def forcing(region: Region, ndays: int, seed: int = 2, doy0: int = 1, day_offset: int = 0):
    """Day-major float32 forcing [ndays, ncell]: precipitation (mm), temperature (C),
    shortwave (W/m2).  Day g of the series (g = day_offset + d) belongs to block
    g // 365, which has its own generator keyed by (seed, block), so a long run can
    be generated piecewise and every piece is the same wherever it is cut."""
    n = region.ncell
    lat = region.lat_deg
    P = np.empty((ndays, n), np.float32)
    T = np.empty((ndays, n), np.float32)
    S = np.empty((ndays, n), np.float32)
    hemi = np.where(lat >= 0, 1.0, -1.0)
    if region.name in ("region_global", "region_5min"):
        tmean = 10.0 + 14.0 * (1.0 - np.abs(lat) / 45.0)
    else:
        tmean = np.full(n, 10.0)
    swamp = np.clip(np.abs(lat) / 30.0, 0.3, 1.0) * hemi
    g0, g1 = day_offset, day_offset + ndays
    for blk in range(g0 // 365, (g1 - 1) // 365 + 1):
        rng = np.random.default_rng((seed, blk))
        u = rng.uniform(size=(365, n))
        amount = rng.gamma(0.8, 8.0, (365, n))
        noise_t = rng.normal(0.0, 3.0, (365, n))
        noise_s = rng.normal(0.0, 10.0, (365, n))
        lo, hi = max(g0, blk * 365), min(g1, (blk + 1) * 365)
        k = np.arange(lo, hi)
        j = k - blk * 365                      # row within the block
        d = k - day_offset                     # row within the output
        doy = (doy0 - 1 + d) % 365 + 1
        P[d] = np.where(u[j] >= 0.6, amount[j], 0.0)
        season = np.sin(2 * np.pi * doy / 365.0)[:, None] * hemi[None, :]
        T[d] = tmean[None, :] + 12.0 * season + noise_t[j]
        sw = 175.0 + 125.0 * np.sin(2 * np.pi * (doy - 80) / 365.0)[:, None] * swamp[None, :]
        S[d] = np.clip(sw + noise_s[j], 50.0, 300.0)
    return P, T, S


def _forcing_year(args):
    factory, seed, y = args
    region = globals()[factory]()
    return forcing(region, 365, seed=seed, doy0=1, day_offset=y * 365)


def forcing_years(factory: str, nyears: int, seed: int = 2, procs: int | None = None):
    """forcing(region, 365 * nyears, seed, doy0=1) of the region that the
    generator `factory` (e.g. "region_global") makes with its defaults, one year
    per spawned worker (safe after a CUDA context exists in the caller); the same
    numbers as one forcing() call."""
    import multiprocessing as mp
    procs = procs or max(1, min(nyears, os.cpu_count() or 1))
    with mp.get_context("spawn").Pool(procs) as pool:
        blocks = pool.map(_forcing_year, [(factory, seed, y) for y in range(nyears)])
    return tuple(np.concatenate([b[k] for b in blocks]) for k in range(3))


def _forcing_chunk(args):
    """Worker of forcing_parallel: cells [c0, c1) of year block blk into shared memory."""
    from multiprocessing import shared_memory
    name, n, c0, c1, seed, blk, lat, tmean_global = args
    shm = shared_memory.SharedMemory(name=name)
    try:
        out = np.ndarray((3, 365, n), np.float32, buffer=shm.buf)
        m = c1 - c0
        rng = np.random.default_rng((seed, blk, c0))
        u = rng.uniform(size=(365, m))
        amount = rng.gamma(0.8, 8.0, (365, m))
        noise_t = rng.normal(0.0, 3.0, (365, m))
        noise_s = rng.normal(0.0, 10.0, (365, m))
        hemi = np.where(lat >= 0, 1.0, -1.0)
        tmean = 10.0 + 14.0 * (1.0 - np.abs(lat) / 45.0) if tmean_global else np.full(m, 10.0)
        swamp = np.clip(np.abs(lat) / 30.0, 0.3, 1.0) * hemi
        doy = np.arange(1, 366)
        out[0, :, c0:c1] = np.where(u >= 0.6, amount, 0.0)
        season = np.sin(2 * np.pi * doy / 365.0)[:, None] * hemi[None, :]
        out[1, :, c0:c1] = tmean[None, :] + 12.0 * season + noise_t
        sw = 175.0 + 125.0 * np.sin(2 * np.pi * (doy - 80) / 365.0)[:, None] * swamp[None, :]
        out[2, :, c0:c1] = np.clip(sw + noise_s, 50.0, 300.0)
    finally:
        shm.close()


def forcing_year_parallel(region: Region, year: int, seed: int = 2, procs: int | None = None, chunk: int = 65536,
                          consume=None):
    """One year (day-of-year 1..365) of forcing [3, 365, ncell] float32 for large
    grids: the distributions of forcing(), with cells split into chunks that
    spawned workers generate in parallel into shared memory, each chunk from its
    own generator keyed by (seed, year, first cell).  The same numbers for any
    worker count.  With consume, the shared array is handed to consume(array)
    instead of being copied out (for grids whose year of forcing is many GB);
    call from a script whose main module can be re-imported (spawned workers)."""
    import multiprocessing as mp
    from multiprocessing import shared_memory
    n = region.ncell
    shm = shared_memory.SharedMemory(create=True, size=3 * 365 * n * 4)
    try:
        lat = region.lat_deg
        glob = region.name in ("region_global", "region_5min")
        jobs = [(shm.name, n, c0, min(n, c0 + chunk), seed, year, lat[c0:min(n, c0 + chunk)], glob)
                for c0 in range(0, n, chunk)]
        with mp.get_context("spawn").Pool(procs or min(len(jobs), os.cpu_count() or 1)) as pool:
            pool.map(_forcing_chunk, jobs)
        view = np.ndarray((3, 365, n), np.float32, buffer=shm.buf)
        if consume is not None:
            consume(view)
            out = None
        else:
            out = view.copy()
        del view
    finally:
        shm.close()
        shm.unlink()
    return out


def water_temp_inputs(region: Region, ndays: int, T: np.ndarray, seed: int = 9):
    """Inputs the water temperature adds to the daily forcing: downward longwave
    radiation [ndays, ncell] float32 (W/m2, from the air temperature through the
    Stefan-Boltzmann law with a seeded effective emissivity), and the yearly
    groundwater temperature [ncell] float32 (the annual mean air temperature of
    the cell plus noise; negative values occur, as in the reference's input)."""
    rng = np.random.default_rng(seed)
    n = region.ncell
    eps = rng.uniform(0.70, 0.95, (ndays, n))
    tk = T.astype(np.float64) + 273.15
    lw = (eps * 5.670374419e-8 * tk ** 4).astype(np.float32)
    gw = (T.astype(np.float64).mean(axis=0) + rng.normal(0.0, 1.5, n)).astype(np.float32)
    return lw, gw


def glwd_units(region: Region) -> np.ndarray:
    """GLWD units (the reference's GLWDunits.UNF4, G_glwdUnit) [ncell] int32, 0 =
    none: the outflow cell of each global lake or reservoir (lake_area or
    res_area > 0), in cell order, gets unit k + 1 together with its riparian
    cells -- the cells draining into it directly and the cell it drains into --
    where those are neither outflow cells nor in an earlier unit.  The riparian
    cells upstream come before the outflow cell in routing order, the one
    downstream after it."""
    n = region.ncell
    unit = np.zeros(n, np.int32)
    outflow = (region.lake_area > 0) | (region.res_area > 0)
    down = region.downstream
    ups = [[] for _ in range(n)]
    for i in range(n):
        if down[i] >= 0:
            ups[down[i]].append(i)
    k = 0
    for c in np.nonzero(outflow)[0]:
        k += 1
        unit[c] = k
        for r in ups[c] + ([int(down[c])] if down[c] >= 0 else []):
            if not outflow[r] and unit[r] == 0:
                unit[r] = k
    return unit


def water_use_inputs(region: Region, nyears: int, seed: int = 13, scale: float = 1.0):
    """Monthly net abstractions as the reference's yearly water-use files hold
    them (m3 per month, float32, [nyears, 12, ncell]): net abstraction from
    surface water (NUs) and from groundwater (NUg), and the withdrawal and
    consumptive use of irrigation from surface water; plus the fraction of
    irrigation return flow that reaches groundwater [ncell] float32.

    About 60 % of the cells use water (lognormal, a few cells far beyond what
    their storages hold, so that demand stays unsatisfied), one in ten of those
    returns water (negative NUs, as return flows make it in the reference's
    input); NUg is negative where irrigation returns more to groundwater than
    is pumped.  Irrigation withdrawal exceeds its consumptive use by the
    efficiency U(0.3, 0.9)."""
    rng = np.random.default_rng(seed)
    n = region.ncell
    area = cell_area_km2(region.row) if region.row is not None else np.full(n, 2500.0)
    users = rng.random(n) < 0.6
    base = rng.lognormal(np.log(2.0e5), 1.6, n) * (area / 2500.0) * scale   # m3 per month
    base[rng.random(n) < 0.03] *= 200.0                                     # unmet demand
    season = 1.0 + 0.6 * np.sin(2.0 * np.pi * (np.arange(12) - 3.0) / 12.0)
    out = []
    for k in range(4):
        noise = rng.lognormal(0.0, 0.3, (nyears, 12, n))
        out.append(base[None, None, :] * season[None, :, None] * noise)
    nus, nug, wdr, _ = out
    sign_s = np.where(rng.random(n) < 0.1, -0.3, 1.0)
    sign_g = np.where(rng.random(n) < 0.25, -0.5, 0.4)
    nus = nus * (users * sign_s)[None, None, :]
    nug = nug * (users * sign_g)[None, None, :]
    irr = users & (rng.random(n) < 0.7)
    wdr = wdr * 1.5 * irr[None, None, :]
    eff = rng.uniform(0.3, 0.9, n)
    cons = wdr * eff[None, None, :]
    frgi = rng.uniform(0.1, 0.9, n).astype(np.float32)
    f32 = lambda a: np.ascontiguousarray(a, np.float32)
    return f32(nus), f32(nug), f32(wdr), f32(cons), frgi
