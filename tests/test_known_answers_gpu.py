"""Known-answer micro cases through the CUDA path: answers derived by hand
from the reference's rules (src/serial/plugin-CLUEClusterizer/CLUEAlgoKernels.h:25-153),
checked against the oracle as well.  Coordinates are chosen so that every
distance involved is exact in fp32 (dyadic differences whose squares and
square roots are exact), which puts points exactly on the <= / > boundaries."""
import numpy as np
import pytest

import clue_gb300 as C
import oracle

from _util import assert_bitexact, assert_bitexact_nan

pytestmark = pytest.mark.gpu
FMAX = np.finfo(np.float32).max


@pytest.fixture(scope="module")
def run(cuda_lib):
    handles = {}

    def go(x, y, layer, w, dc, rhoc, odf):
        key = (dc, rhoc, odf)
        if key not in handles:
            handles[key] = C.Clusterizer(dc, rhoc, odf)
        x, y = np.asarray(x, np.float32), np.asarray(y, np.float32)
        layer, w = np.asarray(layer, np.int32), np.asarray(w, np.float32)
        got = handles[key].make_clusters(x, y, layer, w)
        assert_bitexact(got, oracle.clue2d(x, y, layer, w, dc, rhoc, odf), label=f"{key}")
        return got

    yield go
    for h in handles.values():
        h.close()


def test_single_point(run):
    o = run([1.0], [2.0], [5], [3.0], 1.3, 2.0, 2.0)
    assert o["rho"][0] == np.float32(3.0) and o["nearestHigher"][0] == -1 and o["delta"][0] == FMAX
    assert o["isSeed"][0] == 1 and o["clusterIndex"][0] == 0


def test_rho_equal_to_rhoc_is_a_seed(run):
    # rho >= rhoc (inclusive): weight exactly rhoc seeds; just below it is an outlier
    o = run([0.0, 100.0], [0.0, 0.0], [0, 0], [2.0, np.nextafter(np.float32(2.0), np.float32(0))], 1.0, 2.0, 2.0)
    assert o["isSeed"].tolist() == [1, 0] and o["clusterIndex"].tolist() == [0, -1]


def test_density_boundary_is_inclusive(run):
    # d = 1.25 exactly = dc: each sees the other (<=); equal rho, the larger index is higher
    o = run([10.0, 11.25], [0.0, 0.0], [1, 1], [1.0, 1.0], 1.25, 0.5, 2.0)
    assert o["rho"].tolist() == [1.5, 1.5]
    assert o["nearestHigher"].tolist() == [1, -1] and o["delta"][0] == np.float32(1.25)
    # delta == dc is not > dc: point 0 follows point 1
    assert o["isSeed"].tolist() == [0, 1] and o["clusterIndex"].tolist() == [0, 0]


def test_seed_needs_delta_strictly_above_dc(run):
    # A (w 2) and B (w 1) exactly dc apart: B's delta == dc -> follower of A
    o = run([0.0, 1.25], [0.0, 0.0], [0, 0], [2.0, 1.0], 1.25, 1.0, 2.0)
    assert o["rho"].tolist() == [2.5, 2.0] and o["nearestHigher"].tolist() == [-1, 0]
    assert o["isSeed"].tolist() == [1, 0] and o["clusterIndex"].tolist() == [0, 0]
    # one ulp further apart: no density overlap, B's delta > dc -> its own seed
    xb = np.nextafter(np.float32(1.25), np.float32(2))
    o = run([0.0, xb], [0.0, 0.0], [0, 0], [2.0, 1.0], 1.25, 1.0, 2.0)
    assert o["rho"].tolist() == [2.0, 1.0] and o["nearestHigher"].tolist() == [-1, 0]
    assert o["isSeed"].tolist() == [1, 1] and o["clusterIndex"].tolist() == [0, 1]


def test_equidistant_higher_first_tile_wins(run):
    # the query at x = 50 (tile column 60) has higher neighbours at x = 49 (column 59) and
    # x = 51 (column 60), both 1.0 away: columns are visited in ascending order, so the
    # one at x = 49 wins although its index is larger; between the two neighbours (2.0 =
    # dm apart, inclusive) equal rho makes the larger index the higher one
    o = run([50.0, 51.0, 49.0], [0.0, 0.0, 0.0], [3, 3, 3], [1.0, 5.0, 5.0], 0.5, 0.5, 4.0)
    assert o["nearestHigher"].tolist() == [2, 2, -1]
    assert o["delta"].tolist() == [1.0, 2.0, float(FMAX)]
    # every delta is above dc = 0.5 and every rho at least rhoc: three seeds
    assert o["isSeed"].tolist() == [1, 1, 1] and o["clusterIndex"].tolist() == [0, 1, 2]
    # the same along y: rows are the inner loop, ascending
    o = run([0.0, 0.0, 0.0], [50.0, 51.0, 49.0], [3, 3, 3], [1.0, 5.0, 5.0], 0.5, 0.5, 4.0)
    assert o["nearestHigher"].tolist() == [2, 2, -1]


def test_nearest_higher_beyond_dm_is_none(run):
    # 2.0 + 1 ulp apart with dm = 2: not within dm -> outlier if below rhoc
    x1 = np.nextafter(np.float32(2.0), np.float32(3))
    o = run([0.0, x1], [0.0, 0.0], [0, 0], [5.0, 0.1], 0.5, 1.0, 4.0)
    assert o["nearestHigher"].tolist() == [-1, -1] and o["clusterIndex"].tolist() == [0, -1]


def test_chain_to_an_outlier_stays_unassigned(run):
    # 2 follows 1, 1 is an outlier (rho < rhoc, delta > odf*dc): both stay -1
    o = run([0.0, 9.0, 9.3], [0.0, 0.0, 0.0], [0, 0, 0], [5.0, 0.4, 0.1], 1.0, 1.0, 2.0)
    assert o["nearestHigher"][2] == 1 and o["clusterIndex"].tolist() == [0, -1, -1]


def test_layers_never_interact(run):
    o = run([0.0, 0.0], [0.0, 0.0], [0, 99], [1.0, 1.0], 1.0, 0.5, 2.0)
    assert o["isSeed"].tolist() == [1, 1] and o["clusterIndex"].tolist() == [0, 1]


def test_non_finite_inputs(cuda_lib):
    """NaN and +-inf coordinates and weights against the oracle (which the
    reference pins for NaN and -inf coordinates; a NaN rho has the reference
    index followers[-1], where the oracle and the GPU keep -1)."""
    from clue_gb300 import synthetic as S
    ev = S.toy_event(6, blobs_per_layer=4, noise_per_layer=30)
    rng = np.random.default_rng(4)
    n = ev["x"].size
    k = rng.choice(n, 120, replace=False)
    ev["x"][k[:20]] = np.nan
    ev["y"][k[20:35]] = np.nan
    ev["x"][k[35:45]] = -np.inf
    ev["y"][k[45:55]] = np.inf
    ev["weight"][k[55:75]] = np.nan
    ev["weight"][k[75:90]] = np.inf
    ev["weight"][k[90:100]] = -np.inf
    ev["x"][k[100:120]] = np.float32(3e9)
    algo = C.Clusterizer(1.3, 2.0, 2.0)
    try:
        got = algo.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
        off = np.array([0, n, 2 * n], np.int64)
        cat = {f: np.concatenate([ev[f], ev[f]]) for f in ("x", "y", "layer", "weight")}
        both = algo.run_batch(off, cat["x"], cat["y"], cat["layer"], cat["weight"])
    finally:
        algo.close()
    want = oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], 1.3, 2.0, 2.0)
    assert_bitexact_nan(got, want, label="single event")
    for e in range(2):
        assert_bitexact_nan({f: v[e * n:(e + 1) * n] for f, v in both.items()}, want, label=f"batch event {e}")
