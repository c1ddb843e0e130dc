"""Shared comparison helpers for the parity tests."""
import numpy as np

STORAGES = ["canopy", "soil", "snow", "gw", "river", "loclake", "locwetl", "glolake", "glowetl", "res"]
STATE_KEYS = STORAGES + ["lai_days", "lai_status", "lai_precsum", "rf_loclake", "rf_locwetl", "rf_glolake",
                         "rf_glowetl", "rf_res", "k_release", "laf", "laf_prev", "fswb_next"]


def max_rel_err(a, b, floor_frac=1e-6):
    """Largest relative difference of a from b.  Elements of b smaller than
    floor_frac * max|b| are compared against that floor instead (storages that
    are practically empty, e.g. snapped to zero at 1e-15)."""
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    if a.size == 0:
        return 0.0
    scale = np.max(np.abs(b))
    if scale == 0.0:
        return float(np.max(np.abs(a)))
    den = np.maximum(np.abs(b), floor_frac * scale)
    return float(np.max(np.abs(a - b) / den))


def state_errors(got, ref, keys=STATE_KEYS, mask=None):
    out = {}
    for k in keys:
        g, r = np.asarray(got[k]), np.asarray(ref[k])
        if mask is not None and g.shape == mask.shape:
            g, r = g[mask], r[mask]
        out[k] = max_rel_err(g, r)
    return out


def input_digest(region, *arrays) -> str:
    """SHA-256 over a region's arrays (by name) and further input arrays: the
    fixtures whose inputs are regenerated from their seeds record it, so that a
    generator that draws differently on another host is reported as such."""
    import hashlib
    h = hashlib.sha256()
    for k in sorted(region.arrays):
        h.update(k.encode())
        h.update(np.ascontiguousarray(region.arrays[k]).tobytes())
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def field_sums(state: dict, keys) -> np.ndarray:
    """Exactly rounded sum over all cells of each state field (math.fsum)."""
    import math
    return np.array([math.fsum(np.asarray(state[k], np.float64).ravel().tolist()) for k in keys])


REF_BANDS = 100   # the reference's snow elevation bands (daily.h:122)


def ref_bound() -> float:
    """Bound of the oracle against the reference's own outputs: bit for bit on
    the x86-64 host that made the fixtures (the oracle run with the reference's
    100 bands); elsewhere libm may round a transcendental differently in the
    last place."""
    import platform
    return 0.0 if platform.machine() in ("x86_64", "AMD64") else 1e-12


def rel_err(got, ref) -> float:
    """Largest |got - ref| / |ref| (0/0 counts as 0; no floor)."""
    got = np.asarray(got, np.float64).ravel()
    ref = np.asarray(ref, np.float64).ravel()
    if ref.size == 0:
        return 0.0
    d = np.abs(got - ref)
    same = (d == 0) | (np.isnan(got) & np.isnan(ref))
    return float(np.max(np.where(same, 0.0, d / np.maximum(np.abs(ref), 1e-300))))
