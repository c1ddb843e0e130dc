"""Learned calibration against the reference's bisection, end to end on the GPU:
basins cut from the global drainage tree, training runs of the plain model
batched as FP32 ensemble members, the network trained by the tensor-core
kernels, then both methods calibrate the same basins with the FP64 plain model
as the arbiter.  What the network gains: fewer plain-model calls per basin at the
same 1 % discharge criterion."""
import pytest

pytestmark = pytest.mark.gpu


def test_learned_calibration_needs_fewer_model_calls():
    from watergap2_gb300.calibration import run_workload
    out = run_workload(nbasin=80, lo=20, hi=400, ndays=730, epochs=60, seed=17)
    bis, lrn, sec = out["bisection"], out["learned"], out["secant_without_network"]
    print({k: out[k] for k in ("basins", "cells", "training_runs", "train_loss")}, bis, sec, lrn)
    assert bis["within_1pct"] >= 0.9
    assert lrn["within_1pct"] >= bis["within_1pct"] - 0.02
    assert lrn["calls_per_basin_mean"] < 0.8 * bis["calls_per_basin_mean"]
    # the network's own share of the gain: its first step beats the reference's first move
    assert lrn["calls_per_basin_mean"] < sec["calls_per_basin_mean"]
