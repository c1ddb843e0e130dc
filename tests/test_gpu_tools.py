"""Run-time tools of a context: chunk length, autotuner (device snapshot of the
state around its trials) and CUDA-graph replay of a run.  None of them may
change a result: the FP64 path gives the same bits under every launch shape and
chunk length, and a replayed graph the same bits as the direct calls."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _region_and_forcing(seed, nd, doy0=1):
    from watergap2_gb300 import synthetic as sy
    region = sy.region_small_swb(seed=seed)
    return region, sy.forcing(region, nd, doy0=doy0)


def test_chunk_steps_do_not_change_results():
    from watergap2_gb300.gpu import Model
    region, (P, T, S) = _region_and_forcing(21, 90)
    ref = Model(region, max_days=90)
    q_ref = ref.run(1, P, T, S)
    for steps in (1, 7, 16):
        m = Model(region, max_days=90)
        assert m.chunk_steps(steps) == steps
        assert np.array_equal(m.run(1, P, T, S), q_ref)


def test_autotune_leaves_state_and_results_unchanged():
    from watergap2_gb300.gpu import Model
    nd = 120
    region, (P, T, S) = _region_and_forcing(22, nd)
    plain = Model(region, max_days=nd, record_balance=True)
    plain.upload_forcing(0, P, T, S)
    total = plain.num_steps(nd)
    plain.run_steps(1, 0, nd, 0, 40)
    plain.run_steps(1, 0, nd, 40, total)
    q_ref, b_ref = plain.discharge(0, nd), plain.balance()

    m = Model(region, max_days=nd, record_balance=True)
    m.upload_forcing(0, P, T, S)
    m.run_steps(1, 0, nd, 0, 40)
    st_before = m.get_state()
    res = m.autotune(1, 0, nd, 40, 32)
    assert res["trials"] >= 4 and res["threads"] % 32 == 0 and res["chunk_steps"] >= 1
    st_after = m.get_state()
    for k in st_before:
        assert np.array_equal(st_before[k], st_after[k]), k
    m.run_steps(1, 0, nd, 40, total)
    assert np.array_equal(m.discharge(0, nd), q_ref)
    assert np.array_equal(m.balance(), b_ref)


def test_graph_replay_equals_direct_calls():
    from watergap2_gb300.gpu import Model
    nd = 60
    region, (P, T, S) = _region_and_forcing(23, nd, doy0=100)
    direct = Model(region, max_days=nd)
    direct.upload_forcing(0, P, T, S)
    total = direct.num_steps(nd)
    direct.run_steps(100, 0, nd, 0, total)
    q1 = direct.discharge(0, nd)
    direct.run_steps(100, 0, nd, 0, total)          # a second pass from the state the first left
    q2 = direct.discharge(0, nd)

    g = Model(region, max_days=nd)
    g.upload_forcing(0, P, T, S)
    g.chunk_steps(16)                               # several launch pairs in the graph
    n0 = g.launch_count
    g.graph_capture(100, 0, nd, 0, total)
    assert g.launch_count == n0                     # captured, not run
    g.graph_launch()
    assert np.array_equal(g.discharge(0, nd), q1)
    g.graph_launch()
    assert np.array_equal(g.discharge(0, nd), q2)
    k = -(-total // 16)                             # wavefront launches per pass
    per_pass = 1 + k if g.vertical_overlap() else 2 * k   # + the vertical-ahead launches
    assert g.launch_count - n0 == 2 * per_pass


def test_ensemble_autotune_and_graph():
    """Ensemble: tuned shape and graph replay give the same bits as the default shape."""
    from watergap2_gb300.gpu import Model
    nd, M = 45, 48
    region, (P, T, S) = _region_and_forcing(24, nd, doy0=150)
    pf = np.exp(np.random.default_rng(5).normal(0.0, 0.3, M)).astype(np.float32)
    ref = Model(region, max_days=nd, precision="fp32", members=M, prec_factor=pf)
    q_ref = ref.run(150, P, T, S)

    m = Model(region, max_days=nd, precision="fp32", members=M, prec_factor=pf)
    m.upload_forcing(0, P, T, S)
    total = m.num_steps(nd)
    res = m.autotune(150, 0, nd, 0, min(total, 24))
    assert res["trials"] >= 4
    m.graph_capture(150, 0, nd, 0, total)
    m.graph_launch()
    assert np.array_equal(m.discharge(0, nd), q_ref)


@pytest.mark.parametrize("kd", [1, 5])
def test_ensemble_stream_overlap_same_bits(kd):
    """Ensemble: the next chunk's vertical balance on the second stream, beside
    the wavefront launch of this chunk (the wavefront on all, 3/4 or 1/2 of its
    blocks), gives the same bits as the launches one after the other, with
    short chunks (many launch pairs, the ring reused), across calls, and
    replayed from a CUDA graph."""
    from watergap2_gb300.gpu import Model
    nd, M = 75, 64
    region, (P, T, S) = _region_and_forcing(24, nd, doy0=150)
    pf = np.exp(np.random.default_rng(5).normal(0.0, 0.3, M)).astype(np.float32)
    kw = dict(max_days=nd, precision="fp32", members=M, prec_factor=pf, days_per_step=kd)
    ref = Model(region, **kw)
    assert ref.vertical_overlap() == 0
    q_ref = ref.run(150, P, T, S)
    for frac in (4, 3, 2):
        m = Model(region, **kw)
        assert m.vertical_overlap(True) == 1
        th, blocks, _ = m.launch_shape()
        m.launch_shape(th, max(1, blocks * frac // 4))
        m.chunk_steps(2)
        m.upload_forcing(0, P, T, S)
        total = m.num_steps(nd)
        for lo, hi in ((0, 7), (7, 20), (20, total)):
            m.run_steps(150, 0, nd, lo, hi)
        assert np.array_equal(m.discharge(0, nd), q_ref), frac
    g = Model(region, **kw)
    g.vertical_overlap(True)
    g.chunk_steps(3)
    g.upload_forcing(0, P, T, S)
    g.graph_capture(150, 0, nd, 0, g.num_steps(nd))
    g.graph_launch()
    assert np.array_equal(g.discharge(0, nd), q_ref)


def test_overlapped_uploads_give_the_same_run():
    """Year-by-year forcing on the copy stream, each year uploaded while the
    previous one runs, equals the run with all forcing uploaded first."""
    from watergap2_gb300.gpu import Model
    region, (P, T, S) = _region_and_forcing(25, 3 * 365)
    ref = Model(region, max_days=3 * 365)
    ref.upload_forcing(0, P, T, S)
    total = ref.num_steps(3 * 365)
    ref.run_steps(1, 0, 3 * 365, 0, total)
    q_ref = ref.discharge(0, 3 * 365)

    m = Model(region, max_days=3 * 365)
    m.upload_forcing(0, P[:365], T[:365], S[:365])
    for y in range(3):
        m.run_steps(1, 0, 3 * 365, 365 * y, 365 * (y + 1))
        if y < 2:
            sl = slice(365 * (y + 1), 365 * (y + 2))
            m.upload_forcing(365 * (y + 1), P[sl], T[sl], S[sl], overlap=True)
    m.run_steps(1, 0, 3 * 365, 3 * 365, total)
    assert np.array_equal(m.discharge(0, 3 * 365), q_ref)


def test_inactive_basins_do_not_change_active_ones():
    """wg_set_active_cells: the basins that run give the same bits as in a full run."""
    from watergap2_gb300.gpu import Model
    nd = 90
    region, (P, T, S) = _region_and_forcing(26, nd)
    down = region.downstream
    basin = np.arange(region.ncell)
    for _ in range(region.ncell):                  # follow each cell to its outlet
        nxt = np.where(down[basin] >= 0, down[basin], basin)
        if np.array_equal(nxt, basin):
            break
        basin = nxt
    outlets = np.nonzero(down < 0)[0]
    keep = np.isin(basin, outlets[::2])
    full = Model(region, max_days=nd)
    q_full = full.run(1, P, T, S)
    part = Model(region, max_days=nd)
    part.set_active_cells(keep)
    q_part = part.run(1, P, T, S)
    run_st = np.isin(full.stations, outlets[::2])
    assert run_st.any() and (~run_st).any()
    assert np.array_equal(q_part[:, run_st], q_full[:, run_st])
    assert not np.array_equal(q_part[:, ~run_st], q_full[:, ~run_st])


def test_forcing_from_unf_files_equals_day_major_upload(tmp_path):
    """The reference's yearly climate files (big-endian, cell-major), byte-swapped
    and transposed on the GPU, give the same run as the day-major upload --
    straight and overlapped on the copy stream."""
    from watergap2_gb300 import unf
    from watergap2_gb300.gpu import Model, read_unf
    nd = 2 * 365
    region, (P, T, S) = _region_and_forcing(27, nd)
    n = region.ncell
    ref = Model(region, max_days=nd)
    q_ref = ref.run(1, P, T, S)
    m = Model(region, max_days=nd)
    for y in range(2):
        sl = slice(365 * y, 365 * (y + 1))
        paths = unf.write_climate_year(str(tmp_path), 2000 + y, P[sl], T[sl], S[sl])
        raws = [read_unf(paths[k], n * 365 * 4) for k in ("prec", "temp", "swrad")]
        m.upload_forcing_unf(365 * y, *raws, overlap=(y == 1))
    m.run_days(1, 0, nd)
    assert np.array_equal(m.discharge(0, nd), q_ref)


def test_forcing_from_cell_major_arrays_equals_day_major_upload():
    """The reference's in-memory yearly grids (cell-major native floats, as
    climateYear.G_*_d365 holds them) transposed on the GPU give the same run as
    the day-major upload, straight and overlapped, a year at a time and a part
    of a year (d_first)."""
    from watergap2_gb300.gpu import Model
    nd = 2 * 365
    region, (P, T, S) = _region_and_forcing(29, nd)
    ref = Model(region, max_days=nd)
    q_ref = ref.run(1, P, T, S)
    m = Model(region, max_days=nd)
    for y in range(2):
        sl = slice(365 * y, 365 * (y + 1))
        cm = [np.ascontiguousarray(x[sl].T) for x in (P, T, S)]      # [ncell][365]
        if y == 0:
            m.upload_forcing_cells(0, *cm, d_first=0, ndays=200)
            m.upload_forcing_cells(200, *cm, d_first=200, ndays=165)
        else:
            m.upload_forcing_cells(365, *cm, overlap=True)
    m.run_days(1, 0, nd)
    assert np.array_equal(m.discharge(0, nd), q_ref)


def test_monthly_aggregates_match_daily_outputs():
    """The wavefront's monthly epilogue against the daily outputs: sums of the
    daily discharge of every cell outside inland sinks, their minimum and
    maximum, and the sum of the day-end surface-water and groundwater storage."""
    from watergap2_gb300.gpu import Model
    nd = 75                                            # Jan 1 .. Mar 16: two full months and a part
    region, (P, T, S) = _region_and_forcing(28, nd)
    n = region.ncell
    m = Model(region, max_days=nd, stations=np.arange(n))
    m.monthly_outputs(3, doy_day0=1)
    m.upload_forcing(0, P, T, S)
    stor = np.zeros((nd, n))
    for d in range(nd):                                # per-day API: state after every day
        m.step_vertical(d + 1, d)
        m.step_routing(d + 1, d)
        st = m.get_state()
        stor[d] = st["gw"] + st["river"] + st["loclake"] + st["locwetl"] + st["glolake"] + st["glowetl"] + st["res"]
    q = m.discharge(0, nd)
    bounds = [(0, 31), (31, 59), (59, nd)]
    avail, sto = m.monthly("river_avail"), m.monthly("storage")
    lo, hi = m.monthly("min_avail"), m.monthly("max_avail")
    cro, vel = m.monthly("cell_runoff"), m.monthly("velocity")
    down = region.downstream
    up = np.zeros((nd, n))                             # upstream inflow of every cell and day
    for c in range(n):
        if down[c] >= 0:
            up[:, down[c]] += q[:, c]
    sink = region.ldd < 0
    for k, (a, b) in enumerate(bounds):
        acc_q, acc_s, acc_r = np.zeros(n), np.zeros(n), np.zeros(n)
        for d in range(a, b):                          # day order, as the kernel adds
            acc_q += q[d]
            acc_s += stor[d]
            acc_r += np.where(sink, 0.0, q[d]) - up[d]
        # inland sinks have no river availability: 0, as the reference's reset grids
        assert np.array_equal(avail[k], np.where(sink, 0.0, acc_q))
        assert np.allclose(sto[k], acc_s, rtol=1e-12, atol=0)
        assert np.array_equal(lo[k], np.where(sink, 0.0, q[a:b].min(axis=0)))
        assert np.array_equal(hi[k], np.where(sink, 0.0, q[a:b].max(axis=0)))
        assert np.allclose(cro[k], acc_r, rtol=1e-9, atol=1e-12 * np.abs(acc_q).max())
        assert np.all(np.isfinite(vel[k])) and np.all(vel[k] > 0)


def test_step_flags_equal_grid_barrier():
    """Per-warp step flags and one grid barrier per step give the same bits
    (global grid: many warps, deep drainage)."""
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_global()
    nd = 40
    P, T, S = sy.forcing(region, nd, doy0=200)
    out = []
    for flags in (0, 1):
        m = Model(region, max_days=nd, record_balance=True)
        m.step_sync(flags)
        m.chunk_steps(16)                      # several launches: flags reset per launch
        q = m.run(200, P, T, S)
        out.append((q, m.balance(), m.get_state()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    for k in out[0][2]:
        assert np.array_equal(out[0][2][k], out[1][2][k]), k


@pytest.mark.parametrize("kd", [2, 5])
def test_days_per_step_equal_one_day_steps(kd):
    """Several days per wavefront step (each cell routes kd consecutive days in
    one step) give the same bits as one day per step: discharge, state and water
    balance, with the run split across calls at arbitrary steps."""
    from watergap2_gb300.gpu import Model
    nd = 73                                          # not a multiple of kd
    region, (P, T, S) = _region_and_forcing(29, nd, doy0=300)
    ref = Model(region, max_days=nd, record_balance=True)
    q_ref = ref.run(300, P, T, S)
    m = Model(region, max_days=nd, record_balance=True, days_per_step=kd)
    m.upload_forcing(0, P, T, S)
    total = m.num_steps(nd)
    assert total == -(-nd // kd) + ref.num_steps(nd) - nd
    cuts = [0, 3, 11, total // 2, total]
    for a, b in zip(cuts[:-1], cuts[1:]):
        m.run_steps(300, 0, nd, a, b)
    assert np.array_equal(m.discharge(0, nd), q_ref)
    assert np.array_equal(m.balance(), ref.balance())
    s_ref, s = ref.get_state(), m.get_state()
    for k in s_ref:
        assert np.array_equal(s[k], s_ref[k]), k


def test_days_per_step_global_and_ensemble():
    """Global grid (deep drainage, water bodies) in FP64 with 4 days per step, and
    an FP32 ensemble with 3 days per step, against one day per step."""
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_global()
    nd = 30
    P, T, S = sy.forcing(region, nd, doy0=120)
    q1 = Model(region, max_days=nd).run(120, P, T, S)
    m4 = Model(region, max_days=nd, days_per_step=4)
    m4.chunk_steps(3)                                # several launch pairs
    assert np.array_equal(m4.run(120, P, T, S), q1)
    small, (Ps, Ts, Ss) = _region_and_forcing(30, nd, doy0=120)
    pf = np.exp(np.random.default_rng(7).normal(0.0, 0.3, 40)).astype(np.float32)
    e1 = Model(small, max_days=nd, precision="fp32", members=40, prec_factor=pf).run(120, Ps, Ts, Ss)
    e3 = Model(small, max_days=nd, precision="fp32", members=40, prec_factor=pf, days_per_step=3)
    assert np.array_equal(e3.run(120, Ps, Ts, Ss), e1)


def test_vertical_overlap_equals_separate_launches():
    """Vertical balance computed by extra warps of the previous wavefront launch
    gives the same bits as its own launch before each chunk: discharge, state and
    water balance, with short chunks and the run split across calls."""
    from watergap2_gb300.gpu import Model
    nd = 80
    region, (P, T, S) = _region_and_forcing(31, nd, doy0=40)
    out = []
    for on in (False, True):
        m = Model(region, max_days=nd, record_balance=True)
        assert m.vertical_overlap() > 0                  # on by default for one FP64 member
        m.vertical_overlap(on)
        assert (m.vertical_overlap() > 0) == on
        m.chunk_steps(7)
        m.upload_forcing(0, P, T, S)
        total = m.num_steps(nd)
        for a, b in ((0, 5), (5, 30), (30, total)):
            m.run_steps(40, 0, nd, a, b)
        out.append((m.discharge(0, nd), m.balance(), m.get_state()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    for k in out[0][2]:
        assert np.array_equal(out[0][2][k], out[1][2][k]), k


def test_vertical_overlap_global_grid():
    """Global grid (one block per SM, 14 warps of cells): overlap on and off agree."""
    from watergap2_gb300 import synthetic as sy
    from watergap2_gb300.gpu import Model
    region = sy.region_global()
    nd = 60
    P, T, S = sy.forcing(region, nd, doy0=250)
    q = []
    for on in (False, True):
        m = Model(region, max_days=nd, record_balance=True)
        m.vertical_overlap(on)
        q.append((m.run(250, P, T, S), m.balance()))
    assert np.array_equal(q[0][0], q[1][0])
    assert np.array_equal(q[0][1], q[1][1])
