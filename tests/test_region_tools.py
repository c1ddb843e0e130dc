"""Host-side region helpers: the reference's inflow-direction table (what its
water temperature sums over), option fields that survive copies and the
fixture format."""
import numpy as np

from watergap2_gb300 import synthetic as sy
from watergap2_gb300.region import inflow_cells, load_npz, save_npz


def test_inflow_cells_follow_the_reference_directions(tmp_path):
    region = sy.region_small_swb(seed=21, block_at=(100, 300))
    ic = inflow_cells(region)
    down = region.downstream
    assert ic.shape == (region.ncell, 9)
    assert (ic[:, 4] == -1).all()                         # a cell never flows into itself
    # every upstream cell appears exactly once, in the row of its downstream cell
    m = np.nonzero(down >= 0)[0]
    rows, cols = np.nonzero(ic >= 0)
    assert sorted(ic[rows, cols].tolist()) == sorted(m.tolist())
    assert (down[ic[rows, cols]] == rows).all()
    # direction index 3 * (1 - drow) + (1 + dcol) (rout_prepare.cpp:358-420)
    drow = region.row[ic[rows, cols]].astype(int) - region.row[rows].astype(int)
    dcol = region.col[ic[rows, cols]].astype(int) - region.col[rows].astype(int)
    assert (3 * (1 - drow) + (1 + dcol) == cols).all()


def test_options_survive_copies_and_fixtures(tmp_path):
    region = sy.region_small_swb(seed=5, ny=12, nx=24)
    r1 = region.with_options(frac_routing=1)
    assert r1.frac_routing == 1 and region.frac_routing == 0
    assert r1.lct_tables is region.lct_tables and r1.extras is region.extras
    p = str(tmp_path / "r.npz")
    save_npz(r1, p, x=np.arange(3))
    r2, ex = load_npz(p)
    assert r2.frac_routing == 1 and np.array_equal(ex["x"], np.arange(3))
    for k in region.arrays:
        assert np.array_equal(r2.arrays[k], r1.arrays[k]), k
