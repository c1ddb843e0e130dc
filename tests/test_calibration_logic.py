"""Host logic of the basin calibration (watergap2_gb300/calibration.py) on a
stand-in for the model: Q(gamma, CFA) = CFA * a / (1 + b * gamma), monotone in
gamma as the model's runoff is.  No GPU."""
import numpy as np

from watergap2_gb300 import calibration as cal


class FakeProblem:
    def __init__(self, a, b, target):
        self.a, self.b, self.target_q = a, b, target
        self.static = np.zeros((a.size, 9), np.float32)
        self.pvol = np.full(a.size, 20.0)
        self.calls = 0
        self.call_seconds = 0.0

    @property
    def nbasin(self):
        return self.a.size

    def simulate(self, gamma, cfa, active=None):
        self.calls += 1
        return cfa * self.a / (1.0 + self.b * gamma)


def _problem(n=200, seed=0):
    rng = np.random.default_rng(seed)
    a = rng.uniform(1.0, 10.0, n)
    b = rng.uniform(0.2, 3.0, n)
    g = np.exp(rng.uniform(np.log(0.1), np.log(5.0), n))
    c = rng.uniform(0.5, 1.5, n)
    return FakeProblem(a, b, c * a / (1.0 + b * g))


def test_bisection_reaches_one_percent_or_clamped_cfa():
    p = _problem()
    res = cal.calibrate_bisection(p)
    err = cal.rel_err(res["q"], p.target_q)
    clamped = np.isin(res["cfa"], (cal.CFA_LO, cal.CFA_HI))
    assert np.all((err < cal.TOL) | clamped)
    assert (err < cal.TOL).mean() > 0.95
    assert 2 <= res["calls"].mean() <= 25
    # gamma stays in its range; CFA only moves when gamma ended at a limit or stalled
    assert np.all((res["gamma"] >= cal.GAMMA_LO) & (res["gamma"] <= cal.GAMMA_HI))


def test_bisection_first_steps_follow_the_reference():
    """Call 1 at gamma0; a miss jumps to the limit on the side of the error
    (calibration.cpp:315-349); call 2 inside the bracket halves it."""
    b = cal.Bisection(1.0)
    b.update(q=2.0, qobs=1.0)          # too much discharge: gamma too small
    assert b.gamma == cal.GAMMA_HI and b.low == 1.0
    b.update(q=0.5, qobs=1.0)          # too little at the upper limit
    assert b.high == cal.GAMMA_HI and b.gamma == (1.0 + cal.GAMMA_HI) / 2
    b2 = cal.Bisection(1.0)
    b2.update(q=0.5, qobs=1.0)         # too little: gamma too large
    assert b2.gamma == cal.GAMMA_LO and b2.high == 1.0


class ExactNet:
    """A stand-in network that proposes the exact step for the stand-in model under
    the calibration convention (CFA = 1 when gamma can reach the target, else
    gamma at a limit and CFA for the rest).  The basin is read from input 0,
    which the test sets to the basin index."""

    def __init__(self, p):
        self.p = p

    def forward(self, x):
        idx = x[:, 0].astype(int)
        g, c = np.exp(x[:, 9] * np.log(50.0)), np.exp(x[:, 10])
        a, b = self.p.a[idx], self.p.b[idx]
        qt = c * a / (1 + b * g) * np.exp(x[:, 11])
        g_new = np.clip((a / qt - 1.0) / b, cal.GAMMA_LO, cal.GAMMA_HI)
        c_new = qt * (1 + b * g_new) / a
        out = np.zeros((x.shape[0], 16), np.float32)
        out[:, 0] = np.log(g_new / g)
        out[:, 1] = np.log(c_new / c)
        return out


def test_learned_driver_with_exact_proposals_needs_two_calls():
    p = _problem(n=100, seed=1)
    p.static[:, 0] = np.arange(p.nbasin)
    res = cal.calibrate_learned(p, ExactNet(p))
    err = cal.rel_err(res["q"], p.target_q)
    assert (err < cal.TOL).mean() > 0.97
    assert res["calls"].mean() <= 2.1
    assert not res["fallback"].any()


def test_learned_driver_falls_back_when_proposals_do_not_help():
    p = _problem(n=50, seed=2)

    class Useless:
        def forward(self, x):
            return np.zeros((x.shape[0], 16), np.float32)   # propose the current point again
    res = cal.calibrate_learned(p, Useless())
    err = cal.rel_err(res["q"], p.target_q)
    missed_first = cal.rel_err(p.simulate(np.ones(50), np.ones(50)), p.target_q) >= cal.TOL
    assert res["fallback"][missed_first].all()
    assert (err < cal.TOL).mean() > 0.9


def test_secant_refinement_without_network_beats_bisection_on_a_smooth_model():
    p = _problem(n=200, seed=3)
    bis = cal.calibrate_bisection(p)
    p2 = _problem(n=200, seed=3)
    sec = cal.calibrate_learned(p2, None)
    assert (cal.rel_err(sec["q"], p2.target_q) < cal.TOL).mean() >= (cal.rel_err(bis["q"], p.target_q) < cal.TOL).mean() - 0.01
    assert sec["calls"].mean() < bis["calls"].mean()
