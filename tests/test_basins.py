"""Calibration basins cut from the drainage tree (no GPU): every copied basin is
a tree that drains to its own outlet, holds exactly the cells upstream of the
chosen outlet, and keeps their inputs."""
import numpy as np

from watergap2_gb300 import basins, synthetic as sy


def test_multi_basin_region_copies_each_upstream_tree():
    region = sy.region_64x64(seed=1)
    bs = basins.cut_basins(region, nbasin=12, lo=5, hi=2000, seed=3)
    r = bs.region
    assert r.ncell == bs.sizes.sum() and bs.nbasin == 12
    down = r.downstream
    assert (down < 0).sum() == bs.nbasin                      # one outlet per basin
    assert np.array_equal(np.nonzero(down < 0)[0], bs.outlet_slot)
    # every cell drains to its own basin's outlet, inside its block
    for b in range(bs.nbasin):
        a, e = bs.start[b], bs.start[b + 1]
        blk = down[a:e]
        assert np.all((blk == -1) | ((blk >= a) & (blk < e)))
        # the copied cells are exactly the source cells upstream of the outlet
        src = set(bs.source_cell[a:e].tolist())
        o = bs.outlet_cell[b]
        up = {o}
        frontier = [o]
        sd = region.downstream
        while frontier:
            c = frontier.pop()
            for u in np.nonzero(sd == c)[0]:
                up.add(int(u))
                frontier.append(int(u))
        assert src == up
    # inputs follow the cells
    assert np.array_equal(r.smax, region.smax[bs.source_cell])
    assert np.array_equal(r.param("P_GAMRUN_C"), region.param("P_GAMRUN_C")[bs.source_cell])
    r.subset_order_check()


def test_basin_sizes_follow_the_requested_range():
    region = sy.region_global()
    bs = basins.cut_basins(region, nbasin=200, lo=20, hi=20000, seed=5)
    assert bs.sizes.min() >= 20
    assert bs.sizes.max() <= 9504                             # the largest basin of this tree
    logs = np.log(bs.sizes)
    assert np.log(20) <= np.median(logs) <= np.log(20000)
