"""Randomised parity: parameter sets and point clouds chosen to reach the
rare paths (three- and many-column search boxes, exact distance ties on a
lattice, duplicated points, zero weights, points outside the tile grid,
dense tiles), each compared bit for bit with the oracle through the batched
and the single-event paths."""
import numpy as np
import pytest

import clue_gb300 as C
import oracle

from _util import assert_bitexact

pytestmark = pytest.mark.gpu


def _cloud(rng, kind, n):
    layer = rng.integers(0, 100, n).astype(np.int32)
    if kind == "lattice":
        # coordinates on a 0.5 cm lattice: many exactly equal distances
        x = (rng.integers(-40, 40, n) * 0.5).astype(np.float32)
        y = (rng.integers(-40, 40, n) * 0.5).astype(np.float32)
        layer = rng.integers(0, 4, n).astype(np.int32)
    elif kind == "duplicates":
        base = rng.normal(0, 3, (n // 4, 2)).astype(np.float32)
        pts = base[rng.integers(0, base.shape[0], n)]
        x, y = pts[:, 0].copy(), pts[:, 1].copy()
        layer = rng.integers(0, 3, n).astype(np.int32)
    elif kind == "wide":
        x = rng.uniform(-400, 400, n).astype(np.float32)  # beyond the [-250, 250] grid: clamped bins
        y = rng.uniform(-400, 400, n).astype(np.float32)
    else:  # dense blobs
        c = rng.uniform(-200, 200, (20, 2))
        k = rng.integers(0, 20, n)
        x = (c[k, 0] + rng.normal(0, 1.5, n)).astype(np.float32)
        y = (c[k, 1] + rng.normal(0, 1.5, n)).astype(np.float32)
        layer = rng.integers(0, 10, n).astype(np.int32)
    w = rng.exponential(1.0, n).astype(np.float32)
    w[rng.random(n) < 0.05] = 0.0
    if kind == "lattice":
        w = (rng.integers(1, 4, n) * 0.5).astype(np.float32)  # equal densities too
    return dict(x=x, y=y, layer=layer, weight=w)


CASES = [(kind, seed, order) for kind in ("lattice", "duplicates", "wide", "blobs") for seed in range(3)
         for order in ("random", "layer-sorted")]


@pytest.mark.parametrize("kind,seed,order", CASES, ids=[f"{k}-{s}-{o}" for k, s, o in CASES])
def test_random_clouds_and_parameters(cuda_lib, kind, seed, order):
    """Random layers take the layer-grouping gather; layer-sorted clouds are
    read in place (their in-tile ranks come from the warp groups)."""
    rng = np.random.default_rng(1000 * seed + len(kind))
    dc = float(rng.choice([0.5, 1.3, 2.6, 4.0, 7.5]))
    rhoc = float(rng.uniform(0.5, 10.0))
    odf = float(rng.choice([0.5, 1.0, 2.0, 3.0]))
    evs = [_cloud(rng, kind, int(rng.integers(500, 20000))) for _ in range(3)]
    if order == "layer-sorted":
        evs = [{k: v[np.argsort(e["layer"], kind="stable")] for k, v in e.items()} for e in evs]
    sizes = [e["x"].size for e in evs]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    cat = {k: np.concatenate([e[k] for e in evs]) for k in evs[0]}
    algo = C.Clusterizer(dc, rhoc, odf)
    try:
        got = algo.run_batch(off, cat["x"], cat["y"], cat["layer"], cat["weight"])
        want = oracle.clue2d_batch(off, cat["x"], cat["y"], cat["layer"], cat["weight"], dc, rhoc, odf, n_threads=8)
        assert_bitexact(got, want, label=f"{kind} dc={dc} rhoc={rhoc} odf={odf}")
        one = algo.make_clusters(evs[1]["x"], evs[1]["y"], evs[1]["layer"], evs[1]["weight"])
        assert_bitexact(one, {k: v[off[1]:off[2]] for k, v in want.items()}, label="single event")
    finally:
        algo.close()


CASES3 = list(range(6))


@pytest.mark.parametrize("seed", CASES3)
def test_random_clue3d_parameters(cuda_lib, seed):
    from clue_gb300 import synthetic as S
    rng = np.random.default_rng(77 + seed)
    n_layers = int(rng.choice([50, 94, 100]))
    prm = dict(n_layers=n_layers, density_sibling_layers=int(rng.integers(0, 5)),
               nh_sibling_layers=int(rng.integers(0, 5)), density_on_same_layer=int(rng.integers(0, 2)),
               nh_on_same_layer=int(rng.integers(0, 2)), critical_density=float(rng.uniform(0.1, 2.0)),
               density_xy_distance_sqr=float(rng.choice([1.0, 3.24, 9.0])))
    evs = []
    for e in range(2):
        ev = S.clue3d_event(1000 * seed + e, n_clusters=int(rng.integers(300, 4000)), n_layers=n_layers)
        k = ev["z"].size
        sc = rng.random(k) < 0.3  # scintillator clusters use their own radius
        ev["isSilicon"] = np.where(sc, 0, 1).astype(np.int32)
        ev["radius"] = np.where(sc, rng.uniform(0.5, 4.0, k), ev["radius"]).astype(np.float32)
        edge = rng.random(k) < 0.1  # phi at the wrap
        ev["phi"] = np.where(edge, np.float32(np.pi) * np.sign(ev["phi"]), ev["phi"]).astype(np.float32)
        evs.append(ev)
    b = S.concat3d(evs)
    algo = C.Clusterizer(1.3, 2.0, 2.0)
    try:
        out, nts = algo.run_clue3d(b["offsets"], b, params=prm)
    finally:
        algo.close()
    names = dict(rho="rho", delta_transverse="delta_t", delta_layers="delta_l", nh_layer="nh_layer",
                 nh_index="nh_idx", isSeed="isSeed", tracksterIndex="tracksterIndex")
    for e in range(2):
        s, t = b["offsets"][e], b["offsets"][e + 1]
        want, nt = oracle.clue3d(S.event3d_of(b, e), **prm)
        assert int(nts[e]) == nt
        assert_bitexact({names[k]: v[s:t] for k, v in out.items()}, want,
                        keys=tuple(names.values()), label=f"{prm} event {e}")
