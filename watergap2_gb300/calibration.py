"""Basin calibration of the runoff coefficient gamma and the areal correction
factor CFA against a target long-term mean discharge -- by the reference's
bisection, and by the learned step proposer with the plain model as the arbiter.

Reference: calibGammaClass::findNewGamma (source/calibration.cpp:266-636),
driven by integrate_wghm_ (source/integrateWGHM.cpp:220, 414-442, 970, 1096-1109):
one full model run of the station's basin per step; gamma starts at its
current value, jumps to a limit of [0.1, 5] on the first miss, then halves the
bracket (or doubles / halves gamma while one side of the bracket is open) until
the simulated mean discharge is within 1 % of the observed one; when gamma
sticks at a limit the cell correction factor CFA = Qobs' / Qsim takes the rest.

Here every basin of a BasinSet is calibrated at once: one plain-model call is
one run of the multi-basin region with each basin's (gamma, CFA), so a call
serves every basin still calibrating, and "calls per basin" counts the calls
each basin needed.  The target of a basin is the mean discharge of a run with
hidden true (gamma*, CFA*).  Both methods must end within 1 % of it.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

GAMMA_LO, GAMMA_HI = 0.1, 5.0
CFA_LO, CFA_HI = 0.5, 1.5
TOL = 0.01
SPINUP_DAYS = 365
EVAL_DAYS = 365


@dataclasses.dataclass
class Problem:
    """A multi-basin region on the GPU, its forcing, and the targets."""
    basins: object            # basins.BasinSet
    model: object             # gpu.Model (FP64), snapshot = start state
    static: np.ndarray        # [nbasin, nstatic] basin summaries (MLP inputs)
    target_q: np.ndarray      # [nbasin] target mean discharge
    true_gamma: np.ndarray
    true_cfa: np.ndarray
    ndays: int
    pvol: np.ndarray = None   # [nbasin] mean precipitation volume per day over the basin
    calls: int = 0
    call_seconds: float = 0.0

    @property
    def nbasin(self) -> int:
        return self.basins.nbasin

    def simulate(self, gamma, cfa, active=None) -> np.ndarray:
        """One plain-model call: every basin with its own (gamma, CFA), from the start
        state; returns each basin's mean outlet discharge over the evaluation year.
        With active (per basin), only those basins run (the others' values are stale)."""
        t0 = time.perf_counter()
        m, b = self.model, self.basins.basin_of_cell
        m.set_active_cells(None if active is None else np.asarray(active, bool)[b])
        m.restore_snapshot()
        m.set_calib_param("P_GAMRUN_C", np.asarray(gamma, np.float64)[b])
        m.set_calib_param("P_CFA", np.asarray(cfa, np.float64)[b])
        m.run_steps(1, 0, self.ndays, 0, m.num_steps(self.ndays))
        q = m.discharge(SPINUP_DAYS, EVAL_DAYS).mean(axis=0)
        self.calls += 1
        self.call_seconds += time.perf_counter() - t0
        return q


def basin_statics(basins, P, T, S) -> np.ndarray:
    """Per-basin summaries of forcing and land (the network's static inputs), from
    forcing of the basins' source cells ([days, source cells])."""
    r = basins.region
    b = basins.basin_of_cell
    src = basins.source_cell
    size = np.bincount(b).astype(np.float64)

    def mean(v):
        return np.bincount(b, weights=v) / size
    pm = P.mean(axis=0)[src].astype(np.float64)
    tm = T.mean(axis=0)[src].astype(np.float64)
    frz = (T < 0).mean(axis=0)[src].astype(np.float64)
    sw = S.mean(axis=0)[src].astype(np.float64)
    wb = ((r.loc_lake > 0) | (r.loc_wetl > 0) | (r.lake_area > 0) | (r.res_area > 0) | (r.glo_wetl > 0)).astype(float)
    arid = (r.aindex == 1).astype(float)
    return np.stack([np.log(size) / 10.0, mean(pm) / 5.0, mean(tm) / 20.0, mean(frz), mean(r.smax.astype(float)) / 500.0,
                     mean(r.lai_max.astype(float)) / 6.0, mean(wb), mean(arid), mean(sw) / 300.0], axis=1)


def basin_precip_volume(basins, P) -> np.ndarray:
    """Mean daily precipitation volume of each basin (mm x km2 x 1e-6 = km3), the
    scale of its discharge."""
    r = basins.region
    v = P.mean(axis=0)[basins.source_cell].astype(np.float64) * r.area_km2.astype(np.float64) * 1e-6
    return np.bincount(basins.basin_of_cell, weights=v)


def step_inputs(static, gamma, cfa, q, q_target, pvol) -> np.ndarray:
    """Network inputs of one proposal: statics, the current point, the runoff
    ratios of the current and of the target discharge, and their log ratio."""
    qc, qt = np.maximum(q, 1e-30), np.maximum(q_target, 1e-30)
    ratio = np.clip(np.log(qt / qc), -5.0, 5.0)
    rc = np.clip(np.log(qc / pvol), -10.0, 2.0) / 5.0
    rt = np.clip(np.log(qt / pvol), -10.0, 2.0) / 5.0
    dyn = np.stack([np.log(gamma) / np.log(50.0), np.log(cfa), ratio, rc, rt], axis=1)
    return np.concatenate([static, dyn], axis=1).astype(np.float32)


def rel_err(q, q_target):
    return np.abs(q - q_target) / np.maximum(np.abs(q_target), 1e-30)


# ------------------------------------------------------------------ bisection
class Bisection:
    """findNewGamma for one station (calibration.cpp:266-636), with one evaluation
    period and no water use or upstream inflow, so sumOfDifferences = Qsim - Qobs.
    The reference accepts within 10 % when gamma sticks at a limit (its
    calibStatus 2) and sizes CFA for Qobs x 1.1 (x 0.9); for the 1 % target of
    this workload the correction factor is sized for Qobs itself and refined
    (CFA x Qobs / Qsim) until the basin is within 1 % or CFA is clamped."""

    def __init__(self, gamma0=1.0):
        self.gamma = float(gamma0)
        self.cfa = 1.0
        self.calls = 0
        self.low = -99.0
        self.high = -99.0
        self.diff_old = 0.0
        self.phase = "gamma"
        self.done = False

    def update(self, q, qobs):
        """Result of the run with (self.gamma, self.cfa); sets the next point or done."""
        self.calls += 1
        diff = q - qobs
        crit = abs(diff / qobs) < TOL
        if self.phase == "cfa":
            if crit or self.cfa in (CFA_LO, CFA_HI) or self.calls > 40:
                self.done = True
                return
            self.cfa = float(np.clip(self.cfa * qobs / q, CFA_LO, CFA_HI))
            return
        if crit:
            self.done = True
            return
        old = self.gamma
        new = None
        if self.calls == 1:
            if diff > 0:
                if old >= GAMMA_HI:
                    new = -99.0
                else:
                    self.low, new = old, GAMMA_HI
            else:
                if old <= GAMMA_LO:
                    new = -99.0
                else:
                    self.high, new = old, GAMMA_LO
        else:
            if diff > 0:
                if old == GAMMA_HI:
                    if self.calls == 2:
                        new, self.high = old, GAMMA_HI
                    else:
                        new = -99.0            # gammaCond 2
                elif self.high < 0:
                    self.low, new = old, old * 2.0
                else:
                    self.low = old
                    new = (self.low + self.high) / 2.0
            else:
                if old == GAMMA_LO:
                    if self.calls == 2:
                        new, self.low = old, GAMMA_LO
                    else:
                        new = -99.0            # gammaCond 2
                elif self.low < 0:
                    new, self.high = old / 2.0, old
                else:
                    self.high = old
                    new = (self.low + self.high) / 2.0
        # stop rules of the reference (calibration.cpp:608-613)
        if new > 0 and new < 0.99 * GAMMA_LO and self.calls > 2:
            new = -99.0
        if new > 0 and self.diff_old != 0 and abs(self.diff_old / diff - 1.0) < 1e-4:
            new = -99.0
        self.diff_old = diff
        if new > 0:
            self.gamma = float(min(new, GAMMA_HI))
            return
        # gamma calibration ended outside 1 % (at a limit, cond2, or stalled): the
        # correction factor takes the rest (cellCorrFactor, calibration.cpp:587-594)
        self.phase = "cfa"
        self.cfa = float(np.clip(self.cfa * qobs / q, CFA_LO, CFA_HI))


def calibrate_bisection(prob: Problem, gamma0=1.0, max_calls=60):
    """The reference's procedure for every basin at once; returns final points,
    calls per basin and the discharge of each basin's final point."""
    n = prob.nbasin
    st = [Bisection(gamma0) for _ in range(n)]
    q_final = np.zeros(n)
    for _ in range(max_calls):
        active = [i for i in range(n) if not st[i].done]
        if not active:
            break
        mask = np.zeros(n, bool)
        mask[active] = True
        q = prob.simulate(np.array([s.gamma for s in st]), np.array([s.cfa for s in st]), mask)
        for i in active:
            q_final[i] = q[i]
            st[i].update(q[i], prob.target_q[i])
    return {"gamma": np.array([s.gamma for s in st]), "cfa": np.array([s.cfa for s in st]),
            "calls": np.array([s.calls for s in st]), "q": q_final}


# --------------------------------------------------------- learned proposals
def _secant(pts, q_target):
    """Next (gamma, CFA) from the last two points, secant in (log gamma, log Q / CFA)
    (discharge scales with CFA); gamma beyond its range goes to the limit and CFA
    takes the remaining factor.  None when the two points do not define a slope."""
    (g1, c1, q1), (g2, c2, q2) = pts[-2], pts[-1]
    if q1 <= 0 or q2 <= 0 or g1 == g2:
        return None
    x1, x2 = np.log(g1), np.log(g2)
    if x1 == x2:
        return None
    y1, y2 = np.log(q1 / c1), np.log(q2 / c2)
    m = (y2 - y1) / (x2 - x1)
    if not np.isfinite(m) or abs(m) < 1e-6:
        return None
    yt = np.log(q_target / c2)
    x3 = x2 + (yt - y2) / m
    lo, hi = np.log(GAMMA_LO), np.log(GAMMA_HI)
    if lo <= x3 <= hi:
        return float(np.exp(x3)), c2
    xb = min(max(x3, lo), hi)
    q_b = np.exp(y2 + m * (xb - x2)) * c2       # predicted discharge at the limit, CFA c2
    return float(np.exp(xb)), float(np.clip(c2 * q_target / q_b, CFA_LO, CFA_HI))


def calibrate_learned(prob: Problem, net=None, gamma0=1.0, max_refine=4, max_calls=60):
    """Start at (gamma0, 1).  First step: the network's proposal (dlog gamma,
    dlog CFA) from the basin statics, the current point and the target -- or,
    without a network, the reference's first move (gamma to the limit on the side
    of the error).  Then secant steps on the plain model's own responses.  Every
    point is a plain-model run; within 1 %: done.  A step that does not bring the
    basin closer, or max_refine secant steps without success: the basin falls
    back to bisection started from its best point."""
    n = prob.nbasin
    tq = prob.target_q
    pvol = prob.pvol if prob.pvol is not None else np.ones(n)
    g0, c0 = np.full(n, float(gamma0)), np.ones(n)
    q0 = prob.simulate(g0, c0)
    calls = np.ones(n, np.int64)
    q_final = q0.copy()
    pts = [[(g0[i], 1.0, q0[i])] for i in range(n)]
    best = [0] * n
    done = rel_err(q0, tq) < TOL
    fallback = np.zeros(n, bool)
    refine = np.zeros(n, np.int64)
    bis = [None] * n
    nxt_g, nxt_c = g0.copy(), c0.copy()
    # first step for every basin not yet within 1 %
    first = ~done
    if net is not None and first.any():
        y = net.forward(step_inputs(prob.static[first], g0[first], c0[first], q0[first], tq[first],
                                    pvol[first]))[:, :2]
        nxt_g[first] = np.clip(g0[first] * np.exp(y[:, 0]), GAMMA_LO, GAMMA_HI)
        nxt_c[first] = np.clip(c0[first] * np.exp(y[:, 1]), CFA_LO, CFA_HI)
    else:
        nxt_g[first] = np.where(q0[first] > tq[first], GAMMA_HI, GAMMA_LO)
    for _ in range(max_calls):
        if done.all():
            break
        active = ~done
        q = prob.simulate(nxt_g, nxt_c, active)
        calls[active] += 1
        err = rel_err(q, tq)
        for i in np.nonzero(active)[0]:
            q_final[i] = q[i]
            if fallback[i]:
                bis[i].update(q[i], tq[i])
                done[i] = err[i] < TOL or bis[i].done
                if not done[i]:
                    nxt_g[i], nxt_c[i] = bis[i].gamma, bis[i].cfa
                continue
            pts[i].append((nxt_g[i], nxt_c[i], q[i]))
            if err[i] < TOL:
                done[i] = True
                continue
            gb, cb, qb = pts[i][best[i]]
            if err[i] < rel_err(qb, tq[i]):
                best[i] = len(pts[i]) - 1
            nxt = _secant(pts[i], tq[i]) if refine[i] < max_refine else None
            if nxt is None or (err[i] >= rel_err(qb, tq[i]) and len(pts[i]) > 2):
                gb, cb, qb = pts[i][best[i]]
                fallback[i] = True
                bis[i] = Bisection(gb)
                bis[i].cfa = cb
                bis[i].update(qb, tq[i])     # the start point's run is already known
                q_final[i] = qb
                done[i] = bis[i].done
                nxt_g[i], nxt_c[i] = bis[i].gamma, bis[i].cfa
            else:
                refine[i] += 1
                nxt_g[i], nxt_c[i] = nxt
    final_g = np.array([bis[i].gamma if fallback[i] else pts[i][-1][0] for i in range(n)])
    final_c = np.array([bis[i].cfa if fallback[i] else pts[i][-1][1] for i in range(n)])
    return {"gamma": final_g, "cfa": final_c, "calls": calls, "fallback": fallback, "q": q_final}


# ------------------------------------------------------------- the workload
def training_runs(basins, P_src, T_src, S_src, ndays, launches_a=20, launches_b=5, members=8, seed=61, device=0):
    """Plain-model runs of every basin for the network's training set, batched as
    FP32 ensemble members: launches of type A run gamma (the member factor on a
    gamma of 1) log-uniform over [0.1, 5] with CFA = 1; type B runs gamma at its
    limits with CFA per basin uniform in [0.5, 1.5] -- the points the reference's
    procedure ends on (gamma first; CFA only when gamma sticks at a limit).
    Returns gamma, cfa, q as [nbasin, runs]."""
    from .gpu import Model
    rng = np.random.default_rng(seed)
    nb = basins.nbasin
    b = basins.basin_of_cell
    m = Model(basins.region, max_days=ndays, stations=basins.outlet_slot, precision="fp32", members=members,
              device=device)
    upload_basin_forcing(m, basins, P_src, T_src, S_src)
    m.save_snapshot()
    total = m.num_steps(ndays)
    G, C, Q = [], [], []
    for k in range(launches_a + launches_b):
        if k < launches_a:
            lo, hi = np.log(GAMMA_LO), np.log(GAMMA_HI)
            edges = np.linspace(lo, hi, members + 1)
            gf = np.exp(rng.uniform(edges[:-1], edges[1:])).astype(np.float32)
            cfa_b = np.ones(nb)
        else:
            gf = np.array([GAMMA_LO, GAMMA_HI] * (members // 2), np.float32)
            cfa_b = rng.uniform(CFA_LO, CFA_HI, nb)
        m.restore_snapshot()
        m.set_calib_param("P_GAMRUN_C", np.ones(b.size))
        m.set_calib_param("P_CFA", cfa_b[b])
        m.set_member_factors(None, gf)
        m.run_steps(1, 0, ndays, 0, total)
        q = m.discharge(SPINUP_DAYS, EVAL_DAYS).mean(axis=0)     # [nbasin, members]
        G.append(np.broadcast_to(gf.astype(np.float64), (nb, members)))
        C.append(np.broadcast_to(cfa_b[:, None], (nb, members)))
        Q.append(q)
    del m
    return np.concatenate(G, 1), np.concatenate(C, 1), np.concatenate(Q, 1)


def training_pairs(static, pvol, G, C, Q, pairs_per_basin=400, seed=62):
    """(inputs, steps): from run r1 of a basin to run r2 of the same basin, the
    step (dlog gamma, dlog CFA) given log(Q_r2 / Q_r1)."""
    rng = np.random.default_rng(seed)
    nb, R = Q.shape
    bi = np.repeat(np.arange(nb), pairs_per_basin)
    r1 = rng.integers(0, R, bi.size)
    r2 = rng.integers(0, R, bi.size)
    ok = (r1 != r2) & (Q[bi, r1] > 0) & (Q[bi, r2] > 0)
    bi, r1, r2 = bi[ok], r1[ok], r2[ok]
    x = step_inputs(static[bi], G[bi, r1], C[bi, r1], Q[bi, r1], Q[bi, r2], pvol[bi])
    y = np.stack([np.log(G[bi, r2] / G[bi, r1]), np.log(C[bi, r2] / C[bi, r1])], 1).astype(np.float32)
    return x, y


def upload_basin_forcing(model, basins, P_src, T_src, S_src, block=365):
    """Forcing of the multi-basin region: each cell takes its source cell's series;
    uploaded a block of days at a time."""
    src = basins.source_cell
    nd = P_src.shape[0]
    for d0 in range(0, nd, block):
        sl = slice(d0, min(nd, d0 + block))
        model.upload_forcing(d0, P_src[sl][:, src], T_src[sl][:, src], S_src[sl][:, src])


def run_workload(nbasin=1000, lo=20, hi=20000, ndays=730, seed=71, device=0, epochs=40, log=None):
    """The calibration workload end to end; returns a dict of its measurements."""
    from . import basins as bmod
    from . import synthetic as sy
    from .gpu import Model
    from .mlp import Mlp
    say = log or (lambda *a: None)
    t_all = time.perf_counter()
    src_region = sy.region_global()
    bs = bmod.cut_basins(src_region, nbasin=nbasin, lo=lo, hi=hi, seed=seed)
    P, T, S = sy.forcing(src_region, ndays, seed=seed + 1, doy0=1)
    static = basin_statics(bs, P, T, S)
    pvol = basin_precip_volume(bs, P)
    say(f"basins: {bs.nbasin}, cells {bs.region.ncell}")
    # training set: 200 runs per basin (25 launches x 8 members)
    t0 = time.perf_counter()
    G, C, Q = training_runs(bs, P, T, S, ndays, device=device)
    t_runs = time.perf_counter() - t0
    x, y = training_pairs(static, pvol, G, C, Q)
    say(f"training runs: {G.shape[1]} per basin in {t_runs:.1f} s; pairs {x.shape[0]}")
    t0 = time.perf_counter()
    net = Mlp(device=device, seed=seed)
    loss = net.train(x, y, epochs=epochs, batch=1024, lr=1e-3, seed=seed)
    t_train = time.perf_counter() - t0
    say(f"trained: loss {loss:.4g} in {t_train:.1f} s")
    # the calibration problem: FP64 plain model, hidden true parameters
    rng = np.random.default_rng(seed + 2)
    g_true = np.exp(rng.uniform(np.log(GAMMA_LO), np.log(GAMMA_HI), bs.nbasin))
    c_true = rng.uniform(CFA_LO, CFA_HI, bs.nbasin)
    model = Model(bs.region, max_days=ndays, stations=bs.outlet_slot, device=device)
    upload_basin_forcing(model, bs, P, T, S)
    model.save_snapshot()
    prob = Problem(basins=bs, model=model, static=static, target_q=np.zeros(bs.nbasin), true_gamma=g_true,
                   true_cfa=c_true, ndays=ndays, pvol=pvol)
    prob.target_q = prob.simulate(g_true, c_true)
    out = {"basins": int(bs.nbasin), "cells": int(bs.region.ncell),
           "basin_cells": {"min": int(bs.sizes.min()), "mean": float(bs.sizes.mean()), "max": int(bs.sizes.max())},
           "days_per_call": ndays, "training_runs": int(G.size), "training_pairs": int(x.shape[0]),
           "training_runs_s": t_runs, "train_s": t_train, "train_loss": loss}
    for name, fn in (("bisection", lambda: calibrate_bisection(prob)),
                     ("secant_without_network", lambda: calibrate_learned(prob, None)),
                     ("learned", lambda: calibrate_learned(prob, net))):
        prob.calls, prob.call_seconds = 0, 0.0
        t0 = time.perf_counter()
        res = fn()
        wall = time.perf_counter() - t0
        err = rel_err(res["q"], prob.target_q)
        out[name] = {"calls_per_basin_mean": float(res["calls"].mean()), "calls_per_basin_max": int(res["calls"].max()),
                     "batched_calls": prob.calls, "wall_s": wall, "call_s_mean": prob.call_seconds / max(prob.calls, 1),
                     "calibrations_per_hour": bs.nbasin / wall * 3600.0,
                     "within_1pct": float((err < TOL).mean()), "final_err_max": float(err.max()),
                     "final_err_median": float(np.median(err))}
        if "fallback" in res:
            out[name]["fallback_frac"] = float(res["fallback"].mean())
        say(name, out[name])
    out["total_s"] = time.perf_counter() - t_all
    return out
