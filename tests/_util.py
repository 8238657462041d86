"""Comparison helpers shared by the tests."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KEYS_2D = ("rho", "delta", "nearestHigher", "isSeed", "clusterIndex")
KEYS_3D = ("rho", "delta_t", "delta_l", "nh_layer", "nh_idx", "isSeed", "tracksterIndex")


def golden_2d():
    return sorted(glob.glob(os.path.join(GOLDEN, "clue2d_*.npz")))


def golden_3d():
    return sorted(glob.glob(os.path.join(GOLDEN, "clue3d_*.npz")))


def load_golden_2d(path):
    z = np.load(path)
    ev = {k: z[k] for k in ("x", "y", "layer", "weight")}
    out = {k: z["out_" + k] for k in KEYS_2D}
    return ev, (float(z["dc"]), float(z["rhoc"]), float(z["odf"])), out


def load_golden_3d(path):
    z = np.load(path)
    fields = ("x", "y", "z", "eta", "phi", "r_over_absz", "radius", "layer", "energy", "isSilicon")
    ev = {k: z[k] for k in fields}
    out = {k: z["out_" + k] for k in KEYS_3D}
    prm = eval(str(z["params"]))  # a dict literal written by make_golden.py
    return ev, prm, out, int(z["n_tracksters"])


def max_ulp(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    # map to a monotone integer line
    a = np.where(a < 0, -(a & 0x7fffffff), a)
    b = np.where(b < 0, -(b & 0x7fffffff), b)
    return int(np.max(np.abs(a - b))) if a.size else 0


def assert_bitexact_nan(got, want, keys=KEYS_2D, label=""):
    """assert_bitexact, except that a NaN matches any NaN (the GPU returns
    the canonical NaN, a CPU keeps the input's payload)."""
    g2, w2 = {}, {}
    for k in keys:
        g, w = np.asarray(got[k]), np.asarray(want[k])
        if g.dtype == np.float32:
            both = np.isnan(g) & np.isnan(w)
            g, w = np.where(both, np.float32(0), g), np.where(both, np.float32(0), w)
        g2[k], w2[k] = g, w
    assert_bitexact(g2, w2, keys, label)


def assert_bitexact(got, want, keys=KEYS_2D, label=""):
    """Every output array identical bit for bit; on failure, report the first
    mismatches and the max ULP distance of the float arrays."""
    msgs = []
    for k in keys:
        g = np.asarray(got[k])
        w = np.asarray(want[k])
        assert g.shape == w.shape, f"{label} {k}: shape {g.shape} != {w.shape}"
        gv = g.view(np.int32) if g.dtype == np.float32 else g
        wv = w.view(np.int32) if w.dtype == np.float32 else w
        bad = np.flatnonzero(gv != wv)
        if bad.size:
            extra = f", max ulp {max_ulp(g, w)}" if g.dtype == np.float32 else ""
            i = bad[:5]
            msgs.append(f"{k}: {bad.size} differ{extra}; first at {i.tolist()}: got {g[i].tolist()} want {w[i].tolist()}")
    assert not msgs, f"{label}: " + " | ".join(msgs)
