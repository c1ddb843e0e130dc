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
