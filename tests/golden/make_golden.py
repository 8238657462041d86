"""Writes the golden vectors in tests/golden/ by running the UNMODIFIED
reference serial code (oracle/_ref/libclue_ref.so, built from the reference
tree by oracle/build.py) on small seeded inputs.

The reference's own golden files (data/output/reference/ref_*k_20_25_2.csv)
and toy-detector inputs are downloaded by its build and are not available,
so these fixtures take their place.  Each .npz holds the inputs, the
parameters and the reference outputs; tests compare the oracle and the CUDA
path against them.  Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "heterogeneous-clue_gb300"))

import oracle  # noqa: E402
from clue_gb300 import synthetic as S  # noqa: E402


def _subsample(ev, layers, per_layer, seed):
    rng = np.random.default_rng(seed)
    keep = []
    for l in layers:
        idx = np.flatnonzero(ev["layer"] == l)
        keep.append(np.sort(rng.choice(idx, min(per_layer, idx.size), replace=False)))
    k = np.concatenate(keep)
    return {a: ev[a][k] for a in ("x", "y", "layer", "weight")}


def edge_event():
    """Hand-built cases: a single point, a pair exactly dc apart, equal-rho
    ties, points outside [-250, 250], layer 99, a chain ending at an outlier,
    duplicates, tile-boundary neighbours."""
    pts = []
    # layer 0: isolated point
    pts.append((0.0, 0.0, 0, 1.0))
    # layer 1: two points 1.3 apart (the dc boundary), equal weights -> equal rho tie
    pts += [(10.0, 10.0, 1, 1.0), (11.3, 10.0, 1, 1.0)]
    # layer 2: points straddling the x tile edge at 0 (bin 50) and the y edge
    pts += [(-0.4, 5.0, 2, 2.0), (0.4, 5.0, 2, 1.5), (0.0, 4.9, 2, 1.0), (0.0, 5.1, 2, 3.0)]
    # layer 3: outside the grid, clamped into border tiles
    pts += [(-300.0, -300.0, 3, 5.0), (-299.0, -300.0, 3, 4.0), (400.0, 260.0, 3, 3.0), (251.0, 251.0, 3, 3.0)]
    # layer 99: a seed, a follower chain, a low-density tail beyond the outlier distance
    pts += [(100.0, 100.0, 99, 10.0), (100.5, 100.0, 99, 2.0), (101.0, 100.0, 99, 1.0), (101.5, 100.0, 99, 0.5),
            (107.0, 100.0, 99, 0.3), (108.0, 100.0, 99, 0.2)]
    # layer 50: duplicated coordinates and equal weights
    pts += [(-20.0, -20.0, 50, 1.0)] * 3 + [(-19.0, -20.0, 50, 1.0)]
    # layer 4: equidistant higher neighbours in two tiles (first-wins order)
    pts += [(4.99, 20.0, 4, 0.5), (3.99, 20.0, 4, 3.0), (5.99, 20.0, 4, 3.0)]
    a = np.array(pts, dtype=np.float64)
    return dict(x=a[:, 0].astype(np.float32), y=a[:, 1].astype(np.float32), layer=a[:, 2].astype(np.int32),
                weight=a[:, 3].astype(np.float32))


CASES_2D = [
    ("toy_sub", lambda: _subsample(S.toy_event(12345), range(100), 50, 1), (1.3, 2.0, 2.0)),
    ("hgcal_sub", lambda: _subsample(S.hgcal_event(1000), range(0, 100, 10), 600, 2), (1.3, 2.0, 2.0)),
    ("hgcal_sub_shuffled", lambda: _shuffle(_subsample(S.hgcal_event(1001), range(0, 100, 10), 600, 3), 4),
     (1.3, 2.0, 2.0)),
    ("toy_ref_config", lambda: _subsample(S.toy_event(777), range(0, 100, 10), 1000, 5), (20.0, 25.0, 2.0)),
    ("toy_ref_config_rhoc10", lambda: _subsample(S.toy_event(778), range(0, 100, 10), 1000, 6), (20.0, 10.0, 2.0)),
    ("edge", edge_event, (1.3, 2.0, 2.0)),
    ("edge_wide", edge_event, (3.0, 1.0, 3.0)),
]


def _shuffle(ev, seed):
    p = np.random.default_rng(seed).permutation(ev["x"].size)
    return {k: v[p] for k, v in ev.items()}


def main():
    oracle.ref_lib()  # raises when the reference tree is absent
    for name, make, (dc, rhoc, odf) in CASES_2D:
        ev = make()
        out = oracle.ref_clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], dc, rhoc, odf)
        np.savez_compressed(os.path.join(HERE, f"clue2d_{name}.npz"), dc=np.float32(dc), rhoc=np.float32(rhoc),
                            odf=np.float32(odf), **ev, **{"out_" + k: v for k, v in out.items()})
        print(name, ev["x"].size, "clusters", int(out["clusterIndex"].max()) + 1)
    for name, seed, n, prm in [("default", 11, 3000, {}),
                               ("config4", 12, 3000, dict(density_sibling_layers=2, nh_sibling_layers=2,
                                                          critical_density=0.5))]:
        ev = S.clue3d_event(seed, n_clusters=n, n_layers=94)
        out, nt = oracle.ref_clue3d(ev, **prm)
        np.savez_compressed(os.path.join(HERE, f"clue3d_{name}.npz"), n_tracksters=np.int32(nt),
                            params=np.array(repr(prm)), **ev, **{"out_" + k: v for k, v in out.items()})
        print("3d", name, n, "tracksters", nt)


if __name__ == "__main__":
    main()
