"""Golden records of the reference's water temperature (calcWaterTemp.cpp).

Runs only where the reference sources are present (the build container): it
builds oracle/_ref/wg_ref_wtemp from them (oracle/Makefile, target "ref"),
feeds it seeded random input records that cover every branch of calcWTemp --
each water body present or not, open water and ice cover (new, growing,
melting, frozen through), no-volume cases, cells without a river, inflows from
none to all eight directions, power-plant cooling -- and stores the records with
the reference's 12 outputs, so that tests/test_wtemp_oracle.py can check the C
restatement bit for bit on any machine.

    python tests/golden/make_wtemp_golden.py
"""
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_case  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference's sources (WG_REFERENCE_SOURCE, else the build container's mount)
REF_SOURCE = os.environ.get("WG_REFERENCE_SOURCE") or "/root/reference/source"
REF = os.path.join(ROOT, "oracle", "_ref", "wg_ref_wtemp")
NIN = 73
# field offsets of a record (calcWaterTempClass::transfer order)
FIELDS = [("pp", 1), ("ww", 1), ("wc", 1), ("sw", 1), ("lw", 1), ("ta", 1), ("cfa", 1), ("owpet", 1),
          ("owprec", 1), ("area", 1), ("tgw", 1), ("inflow", 9), ("inflow_t", 9), ("ice", 6),
          ("rstor", 1), ("gw_ir", 1), ("r_ir", 1), ("bw", 1), ("rlen", 1), ("rlen_chk", 1), ("rin", 1),
          ("has_out", 1),
          ("ll_area", 1), ("ll_stor", 1), ("ll_t", 1), ("ll_ev", 1), ("ll_rf", 1), ("lrun", 1), ("lgw", 1),
          ("lw_area", 1), ("lw_stor", 1), ("lw_t", 1), ("lw_ev", 1), ("lw_rf", 1), ("lw_in", 1), ("lw_out", 1),
          ("gl_area", 1), ("gl_stor", 1), ("gl_t", 1), ("gl_ev", 1), ("gl_in", 1),
          ("rs_in", 1), ("rs_area", 1), ("rs_stor", 1), ("rs_t", 1), ("rs_ev", 1),
          ("gw_in", 1), ("gw_area", 1), ("gw_stor", 1), ("gw_t", 1), ("gw_ev", 1), ("gw_rf", 1)]
F = {}
_o = 0
for _name, _w in FIELDS:
    F[_name] = (_o, _o + _w)
    _o += _w
assert max(v[1] for v in F.values()) == NIN


def records(n, seed=7):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, NIN))

    def put(name, v):
        a, b = F[name]
        r[:, a:b] = np.asarray(v).reshape(n, b - a) if b - a > 1 else np.asarray(v).reshape(n, 1)

    u = rng.random
    cold = u(n) < 0.45
    ta = np.where(cold, rng.uniform(-30, 2, n), rng.uniform(-2, 38, n))
    ta[u(n) < 0.03] = 0.0
    put("ta", ta)
    put("sw", rng.uniform(0, 350, n))
    put("lw", rng.uniform(150, 450, n))
    put("cfa", np.where(u(n) < 0.5, 1.0, rng.uniform(0.5, 1.5, n)))
    put("owprec", np.where(u(n) < 0.5, 0.0, rng.gamma(0.8, 8, n)))
    put("owpet", rng.uniform(0, 8, n))
    cell_area = rng.uniform(500, 3000, n)
    put("area", cell_area)
    put("tgw", rng.uniform(0, 25, n))
    # inflows by direction; the cell itself (index 4) carries no volume
    present = u((n, 9)) < rng.uniform(0, 0.6, (n, 1))
    present[:, 4] = False
    vol = np.where(present, rng.lognormal(-7, 2, (n, 9)), 0.0)
    put("inflow", vol)
    put("inflow_t", np.where(present | (np.arange(9) == 4), rng.uniform(0, 30, (n, 9)), 15.0))

    def ice_of(p):
        # no ice, thin, thick, or a record of an absent water body
        k = rng.integers(0, 4, n)
        return np.select([k == 0, k == 1, k == 2], [0.0, rng.uniform(1e-7, 5e-6, n), rng.uniform(5e-6, 2e-3, n)],
                         -9999.0 * (p == 0))
    has = {k: u(n) < p for k, p in [("ll", 0.4), ("lw", 0.4), ("gl", 0.3), ("rs", 0.3), ("gw", 0.3)]}
    ices = np.stack([ice_of(np.ones(n))] + [ice_of(has[k]) for k in ("ll", "lw", "gl", "rs", "gw")], axis=1)
    put("ice", np.where(u((n, 6)) < 0.15, 0.0, ices))
    # river
    rlen = rng.uniform(20, 200, n)
    put("rlen", rlen)
    put("rlen_chk", np.where(u(n) < 0.15, 55.0, rlen * rng.uniform(0.5, 1.0, n)))
    put("has_out", (u(n) < 0.85).astype(float))
    rstor = np.where(u(n) < 0.1, 0.0, rng.lognormal(-5, 2, n))
    put("rstor", rstor)
    put("bw", rng.uniform(1, 400, n))
    put("rin", np.where(u(n) < 0.2, 0.0, rng.lognormal(-6, 2, n)))
    into = u(n) < 0.2
    put("r_ir", np.where(into, rng.lognormal(-8, 1, n), 0.0))
    put("gw_ir", np.where(into, rng.lognormal(-9, 1, n), 0.0))
    lgw = np.where(u(n) < 0.2, 0.0, rng.lognormal(-8, 1.5, n))
    put("lgw", lgw)
    put("lrun", lgw + np.where(u(n) < 0.3, 0.0, rng.lognormal(-8, 1.5, n)))

    def swb(prefix, pct_area, stor_scale):
        area = np.where(has[prefix], pct_area, 0.0)
        put(f"{prefix}_area", area)
        st = rng.lognormal(np.log(stor_scale), 1.5, n)
        st[u(n) < 0.08] = 0.0
        st[u(n) < 0.04] = 1e-12                      # nearly empty: frozen through
        put(f"{prefix}_stor", st)
        put(f"{prefix}_t", np.where(u(n) < 0.2, 0.0, rng.uniform(0, 30, n)))
        put(f"{prefix}_ev", rng.uniform(0, 6, n))
    swb("ll", rng.uniform(0.1, 20, n), 1e-2)
    put("ll_rf", rng.uniform(0.2, 1, n))
    swb("lw", rng.uniform(0.1, 20, n), 1e-3)
    put("lw_rf", rng.uniform(0.2, 1, n))
    put("lw_in", np.where(has["ll"] & (u(n) < 0.8), rng.lognormal(-8, 2, n), 0.0))
    put("lw_out", np.where(has["lw"] & (u(n) < 0.8), rng.lognormal(-8, 2, n), 0.0))
    swb("gl", rng.uniform(5, 2000, n), 1.0)
    put("gl_in", rng.lognormal(-6, 2, n))
    swb("rs", rng.uniform(5, 500, n), 0.5)
    put("rs_in", rng.lognormal(-6, 2, n))
    swb("gw", rng.uniform(0.1, 30, n), 1e-2)
    put("gw_rf", rng.uniform(0.2, 1, n))
    put("gw_in", rng.lognormal(-6, 2, n))
    pp = u(n) < 0.1
    put("pp", pp.astype(float))
    put("ww", np.where(pp, rng.lognormal(-6, 2, n), 0.0))
    put("wc", np.where(pp, rng.lognormal(-8, 2, n), 0.0))
    return r


def main(n=2000):
    if not os.path.exists(REF):
        if not ref_case.build(REF_SOURCE):
            raise SystemExit("reference sources not found; cannot regenerate fixtures")
    rec = records(n)
    out = subprocess.run([REF], input=rec.astype("<f8").tobytes(), stdout=subprocess.PIPE, check=True).stdout
    res = np.frombuffer(out, "<f8").reshape(n, 12)
    path = os.path.join(HERE, "wtemp_cases.npz")
    np.savez_compressed(path, records=rec, out=res)
    t = res[:, :6]
    print(f"wtemp_cases: {n} records -> {os.path.getsize(path) / 1e6:.2f} MB; "
          f"no temperature {np.mean(t == -9999.):.2f}, zero {np.mean(t == 0):.2f}, ice {np.mean(res[:, 6:] > 0):.2f}")


if __name__ == "__main__":
    main()
