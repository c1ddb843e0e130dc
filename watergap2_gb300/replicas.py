"""Several GPUs: one process per GPU, no collective in the data path.

The daily step has no exchange between drainage basins (the reference's
water-use couplings that would connect them are off on this path), so the
work shards without communication:

* replicas -- every rank runs the whole workload on its own GPU (the bench's
  weak-scaling mode: the work per GPU is fixed as N grows);
* basin shards -- the drainage basins (outlet trees) are split over the ranks
  by longest-processing-time bin packing on their cell counts, each rank runs
  the region of its basins.

The only collectives are on the host side of the measurement: a barrier around
the timed region and the maximum of the ranks' elapsed times.
"""
from __future__ import annotations

import numpy as np

from .region import FIELDS, NPARAM, Region


def job_seconds(seconds: float, dist=None, device=None) -> float:
    """The job's elapsed time: the maximum over the ranks of each rank's own
    (the slowest rank ends the job); without a process group, the rank's own."""
    if dist is None:
        return float(seconds)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Throughput of the whole job: all ranks' units over the slowest rank's time."""
    return float(units_per_rank) * world / seconds_max


def basin_of(region: Region) -> np.ndarray:
    """The outlet (basin) of every cell."""
    down = region.downstream
    basin = np.arange(region.ncell)
    for _ in range(region.ncell):
        nxt = np.where(down[basin] >= 0, down[basin], basin)
        if np.array_equal(nxt, basin):
            return basin
        basin = nxt
    raise ValueError("drainage graph has a cycle")


def shard_basins(region: Region, world: int) -> list:
    """Basin outlets of each rank: largest basin first onto the rank with the
    fewest cells so far (LPT); returns [world] arrays of outlet cells."""
    basin = basin_of(region)
    outlets, size = np.unique(basin, return_counts=True)
    load = np.zeros(world, np.int64)
    share = [[] for _ in range(world)]
    for k in np.argsort(-size, kind="stable"):
        r = int(np.argmin(load))
        share[r].append(int(outlets[k]))
        load[r] += size[k]
    return [np.array(sorted(s), np.int64) for s in share]


def basin_region(region: Region, outlets) -> tuple:
    """The region of the given basins: their cells in the source order, the
    source routing order restricted to them (so every confluence sums in the
    same order), downstream links renumbered.  Returns (region, source cells)."""
    basin = basin_of(region)
    keep = np.isin(basin, np.asarray(outlets))
    src = np.nonzero(keep)[0]
    new_of = -np.ones(region.ncell, np.int64)
    new_of[src] = np.arange(src.size)
    n = src.size
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
    d = region.downstream[src]
    arrays["downstream"] = np.where(d >= 0, new_of[np.maximum(d, 0)], -1).astype(region.downstream.dtype)
    order = region.rout_order[keep[region.rout_order]]
    arrays["rout_order"] = new_of[order].astype(region.rout_order.dtype)
    out = region.with_options(ncell=int(n), arrays=arrays, name=f"{region.name}_shard",
                              row=None if region.row is None else region.row[src],
                              col=None if region.col is None else region.col[src])
    if "extras" in region.__dict__:
        out.__dict__["extras"] = {k: (v[src] if isinstance(v, np.ndarray) and v.shape[:1] == (region.ncell,) else v)
                                  for k, v in region.__dict__["extras"].items()}
    return out, src
