"""Time the reference's own calcNewDay/routing object code against the C
restatement (the CPU baseline), where the reference sources exist.

TEST AND MEASUREMENT INFRASTRUCTURE ONLY.  Runs the harness
(oracle/_ref/wg_ref_harness, built from the reference's sources by ``make
ref``) and the oracle port on the same seeded workloads -- the 64 x 64 region
over a year and the 67,420-cell global grid with water bodies over a bounded
window -- with the vertical pass on 1 thread and on every host thread (the
reference's OpenMP cell loop, integrateWGHM.cpp:767-783) and routing serial (as
the reference runs it, routing.cpp:1830-1835).  Reports cell-days/s of the
vertical pass, of routing and of the whole day, and the port/reference ratio.
File writing and reading are outside the timed passes.  Both run the reference's
100 snow bands (the port with the 5 synthetic bands replicated 20 times), so the
two do the same arithmetic.

    python oracle/time_reference.py [global_days]
"""
from __future__ import annotations

import json
import os
import platform
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def _rates(ncell, ndays, vertical_s, routing_s):
    cd = ncell * ndays
    return {"vertical_cell_days_per_s": cd / vertical_s, "routing_cell_days_per_s": cd / routing_s,
            "total_cell_days_per_s": cd / (vertical_s + routing_s), "vertical_s": vertical_s,
            "routing_s": routing_s}


def time_case(name, region, ndays, threads_list):
    from oracle import Oracle, ref_case
    from watergap2_gb300 import synthetic as sy
    P, T, S = sy.forcing(region, ndays, seed=2, doy0=1)
    out = {"workload": name, "ncell": region.ncell, "days": ndays, "runs": []}
    reg100 = region.with_bands(ref_case.REF_BANDS)
    for th in threads_list:
        r = ref_case.run(region, P, T, S, doy0=1, threads=th)
        ref = _rates(region.ncell, ndays, r["timing"]["vertical_s"], r["timing"]["routing_s"])
        o = Oracle(reg100)
        t0 = time.perf_counter()
        o.run(1, P, T, S, nthreads=th)
        wall = time.perf_counter() - t0
        tm = Oracle.last_timing()
        port = _rates(region.ncell, ndays, tm["vertical_s"], tm["routing_s"])
        port["wall_s"] = wall
        out["runs"].append({"threads": th, "reference": ref, "port": port,
                            "port_over_reference": port["total_cell_days_per_s"] / ref["total_cell_days_per_s"]})
    return out


def main(global_days: int = 60):
    from oracle import ref_case
    from watergap2_gb300 import synthetic as sy
    if not ref_case.available():
        src = os.environ.get("WG_REFERENCE_SOURCE")
        if not ref_case.build(src):
            raise SystemExit("reference harness not built and WG_REFERENCE_SOURCE not set")
    threads = sorted({1, os.cpu_count() or 1})
    res = {"host": {"cpu": _cpu_model(), "nproc": os.cpu_count(), "machine": platform.machine()},
           "cases": [time_case("64 x 64 region, no water bodies, 365 days", sy.region_64x64(), 365, threads),
                     time_case(f"global 0.5-degree grid, 67,420 cells, water bodies, {global_days} days",
                               sy.region_global(), global_days, threads)]}
    print(json.dumps(res, indent=1))
    return res


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 60)
