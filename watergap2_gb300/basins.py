"""Calibration basins cut from a drainage tree, and the multi-basin region that
simulates all of them in one context.

The reference calibrates one gauged basin at a time: the cells upstream of the
station are flagged (G_toBeCalculated, source/integrateWGHM.cpp:421-442) and
the whole model is run for them once per bisection step.  Here every basin is
an independent copy of its cells in one region (a forest of basin trees, each
basin outlet a region outlet), so one run of the context is one model run of
every basin, each with its own gamma and correction factor (wg_set_calib_param).
Nested basins share no state: a cell upstream of two chosen outlets is copied
into both.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .region import FIELDS, NPARAM, Region


def dfs_order(downstream: np.ndarray):
    """Depth-first (pre-order) numbering of the drainage forest: every subtree --
    the basin upstream of a cell -- is the contiguous range tin[c]..tout[c]."""
    n = downstream.size
    children = [[] for _ in range(n)]
    roots = []
    for c in range(n):
        d = int(downstream[c])
        if d >= 0:
            children[d].append(c)
        else:
            roots.append(c)
    order = np.empty(n, np.int64)
    tin = np.empty(n, np.int64)
    tout = np.empty(n, np.int64)
    k = 0
    for r in roots:
        stack = [(r, 0)]
        while stack:
            c, i = stack.pop()
            if i == 0:
                tin[c] = k
                order[k] = c
                k += 1
            if i < len(children[c]):
                stack.append((c, i + 1))
                stack.append((children[c][i], 0))
            else:
                tout[c] = k - 1
    assert k == n
    return order, tin, tout


@dataclasses.dataclass
class BasinSet:
    region: Region              # the multi-basin region
    outlet_cell: np.ndarray     # [nbasin] outlet cell of each basin in the source region
    start: np.ndarray           # [nbasin + 1] first cell of each basin in the multi-basin region
    basin_of_cell: np.ndarray   # [ncell] basin index of each multi-basin cell
    outlet_slot: np.ndarray     # [nbasin] cell index of each basin's outlet in the multi-basin region
    source_cell: np.ndarray     # [ncell] cell of the source region each cell copies

    @property
    def nbasin(self) -> int:
        return self.outlet_cell.size

    @property
    def sizes(self) -> np.ndarray:
        return np.diff(self.start)


def cut_basins(region: Region, nbasin: int = 1000, lo: int = 20, hi: int = 20000, seed: int = 51) -> BasinSet:
    """nbasin basins whose cell counts are drawn log-uniform from [lo, hi]: for each
    draw, the outlet is a cell whose upstream area is the nearest available (ties
    broken at random); draws above the largest basin of the tree take the largest
    ones.  Returns the multi-basin region (cells copied per basin, in depth-first
    order, each basin outlet a region outlet)."""
    rng = np.random.default_rng(seed)
    order, tin, tout = dfs_order(region.downstream)
    area = tout - tin + 1
    by_area = np.argsort(area, kind="stable")
    sorted_area = area[by_area]
    want = np.exp(rng.uniform(np.log(lo), np.log(hi), nbasin))
    outlets = np.empty(nbasin, np.int64)
    for b, w in enumerate(want):
        j = int(np.searchsorted(sorted_area, w))
        j = min(max(j, 0), sorted_area.size - 1)
        if j > 0 and abs(sorted_area[j - 1] - w) < abs(sorted_area[j] - w):
            j -= 1
        same = np.nonzero(sorted_area == sorted_area[j])[0]
        outlets[b] = by_area[rng.choice(same)]
    return multi_basin_region(region, outlets, order, tin, tout)


def multi_basin_region(region: Region, outlets: np.ndarray, order=None, tin=None, tout=None) -> BasinSet:
    if order is None:
        order, tin, tout = dfs_order(region.downstream)
    sizes = tout[outlets] - tin[outlets] + 1
    start = np.concatenate([[0], np.cumsum(sizes)])
    src = np.concatenate([order[tin[o]:tout[o] + 1] for o in outlets])
    n = src.size
    basin = np.repeat(np.arange(outlets.size), sizes)
    # downstream inside the copy: the same offset from the basin's first cell
    d_old = region.downstream[src]
    base_old = tin[outlets][basin]
    down = np.where(d_old >= 0, start[basin] + (tin[np.maximum(d_old, 0)] - base_old), -1)
    down[start[:-1]] = -1                      # each basin outlet drains out of the region
    arrays = {}
    nb1 = region.nband + 1
    for name, _, per in FIELDS:
        arr = region.arrays[name]
        if per == "cell":
            arrays[name] = arr[src]
        elif per == "band":
            arrays[name] = arr.reshape(region.ncell, nb1)[src].reshape(-1)
        elif per == "param":
            arrays[name] = arr.reshape(NPARAM, region.ncell)[:, src].reshape(-1)
        else:
            arrays[name] = arr
    arrays["downstream"] = down.astype(region.downstream.dtype)
    arrays["rout_order"] = _upstream_first(down).astype(region.rout_order.dtype)
    out = dataclasses.replace(region, ncell=int(n), arrays=arrays, name=f"{region.name}_basins",
                              row=None if region.row is None else region.row[src],
                              col=None if region.col is None else region.col[src])
    for k in ("lct_tables", "extras"):
        if k in region.__dict__:
            out.__dict__[k] = region.__dict__[k]
    return BasinSet(region=out, outlet_cell=np.asarray(outlets), start=start, basin_of_cell=basin,
                    outlet_slot=start[:-1].copy(), source_cell=src)


def _upstream_first(down: np.ndarray) -> np.ndarray:
    """A routing order (every cell before its downstream cell): Kahn passes in
    index order, as the reference's rout_order (source/rout_prepare.cpp:834-886)."""
    n = down.size
    cnt = np.zeros(n, np.int64)
    m = down >= 0
    np.add.at(cnt, down[m], 1)
    frontier = np.nonzero(cnt == 0)[0]
    out = []
    while frontier.size:
        out.append(frontier)
        d = down[frontier]
        d = d[d >= 0]
        np.subtract.at(cnt, d, 1)
        frontier = np.unique(d[cnt[d] == 0])
    res = np.concatenate(out)
    assert res.size == n
    return res
