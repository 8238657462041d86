"""The oracle (CPU restatement) pinned against the reference: the golden
vectors written by the unmodified serial code, and -- where the reference
tree is present -- the reference itself on fresh seeded inputs."""
import numpy as np
import pytest

import oracle
from clue_gb300 import synthetic as S

from _util import KEYS_3D, assert_bitexact, golden_2d, golden_3d, load_golden_2d, load_golden_3d

needs_ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not present")


@pytest.mark.parametrize("path", golden_2d(), ids=lambda p: p.split("/")[-1])
def test_oracle_matches_golden_2d(path):
    ev, prm, want = load_golden_2d(path)
    got = oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *prm)
    assert_bitexact(got, want, label=path)


@pytest.mark.parametrize("path", golden_3d(), ids=lambda p: p.split("/")[-1])
def test_oracle_matches_golden_3d(path):
    ev, prm, want, nt = load_golden_3d(path)
    got, nt2 = oracle.clue3d(ev, **prm)
    assert nt2 == nt
    assert_bitexact(got, want, KEYS_3D, label=path)


@needs_ref
@pytest.mark.parametrize("seed,prm,shuffle", [(12345, (1.3, 2.0, 2.0), False), (4, (1.3, 2.0, 2.0), True),
                                              (5, (20.0, 25.0, 2.0), False), (6, (2.0, 3.0, 1.2), False),
                                              (7, (0.7, 1.0, 4.0), True)])
def test_oracle_matches_reference_toy(seed, prm, shuffle):
    ev = S.toy_event(seed, shuffle=shuffle)
    assert_bitexact(oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *prm),
                    oracle.ref_clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *prm), label=str(prm))


@needs_ref
def test_oracle_matches_reference_hgcal():
    ev = S.hgcal_event(1000)
    prm = (1.3, 2.0, 2.0)
    assert_bitexact(oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *prm),
                    oracle.ref_clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *prm))


@needs_ref
@pytest.mark.parametrize("seed", [1, 2])
@pytest.mark.parametrize("prm", [{}, dict(density_sibling_layers=2, nh_sibling_layers=2, critical_density=0.5),
                                 dict(density_on_same_layer=1, nh_on_same_layer=1, kernel_density_factor=0.5)])
def test_oracle_matches_reference_3d(seed, prm):
    ev = S.clue3d_event(seed, n_layers=94)
    got, nt = oracle.clue3d(ev, **prm)
    want, nt2 = oracle.ref_clue3d(ev, **prm)
    assert nt == nt2
    assert_bitexact(got, want, KEYS_3D)


@needs_ref
def test_oracle_matches_reference_3d_scintillator_and_wrap():
    """Non-silicon clusters (radius thresholds) and phi near +-pi."""
    ev = S.clue3d_event(3, n_clusters=4000, n_layers=94)
    rng = np.random.default_rng(0)
    ev["isSilicon"] = (rng.random(ev["z"].size) < 0.5).astype(np.int32)
    ev["radius"] = rng.uniform(0.5, 3.0, ev["z"].size).astype(np.float32)
    ev["phi"][:500] = np.float32(np.pi) - rng.uniform(0, 0.05, 500).astype(np.float32)
    ev["phi"][500:1000] = -np.float32(np.pi) + rng.uniform(0, 0.05, 500).astype(np.float32)
    got, nt = oracle.clue3d(ev)
    want, nt2 = oracle.ref_clue3d(ev)
    assert nt == nt2
    assert_bitexact(got, want, KEYS_3D)


@needs_ref
@pytest.mark.parametrize("prm", [{}, dict(density_sibling_layers=2, nh_sibling_layers=2, critical_density=0.5)])
def test_oracle_3d_side_boundary_and_high_eta_on_the_reference(prm):
    """Dense clusters on layers 44-51 only, around the detector sides' split
    (density windows stop below layer 47, the upper nearest-higher window
    starts at 48 with 94 layers), with eta up to 3.0 (the last eta rows) and
    phi in a narrow band: every cluster's windows cross the boundary."""
    rng = np.random.default_rng(11)
    ev = S.clue3d_event(12, n_clusters=3000, n_layers=94, eta_range=(2.8, 3.0))
    layer = rng.integers(44, 52, ev["z"].size).astype(np.int32)
    phi = rng.uniform(0.0, 0.4, ev["z"].size).astype(np.float32)
    z = S.layer_z(94)[layer].astype(np.float32)
    r = ev["r_over_absz"] * z
    ev.update(layer=layer, phi=phi, z=z, x=(r * np.cos(phi)).astype(np.float32), y=(r * np.sin(phi)).astype(np.float32))
    got, nt = oracle.clue3d(ev, **prm)
    want, nt2 = oracle.ref_clue3d(ev, **prm)
    assert nt == nt2
    assert_bitexact(got, want, KEYS_3D)


def test_oracle_known_answers():
    """Hand-derived answers for a few micro cases."""
    # one point: rho = own weight, no higher, seed iff rho >= rhoc
    o = oracle.clue2d([1.0], [2.0], [5], [3.0], 1.3, 2.0, 2.0)
    assert o["rho"][0] == np.float32(3.0) and o["nearestHigher"][0] == -1
    assert o["delta"][0] == np.finfo(np.float32).max and o["isSeed"][0] == 1 and o["clusterIndex"][0] == 0
    # two points exactly dc apart in x (1.3 is representable as the float difference below)
    x = np.array([10.0, 11.3], np.float32)
    d = np.float32(np.sqrt(np.float32(x[1] - x[0]) ** 2))
    o = oracle.clue2d(x, [0.0, 0.0], [1, 1], [1.0, 1.0], float(d), 0.5, 2.0)
    # inside dc (<=): rho = 1 + 0.5; equal rho, j > i wins: point 0 follows point 1
    assert o["rho"].tolist() == [1.5, 1.5]
    assert o["nearestHigher"].tolist() == [1, -1]
    assert o["isSeed"].tolist() == [0, 1] and o["clusterIndex"].tolist() == [0, 0]
    # a low-density point beyond odf*dc of anything is an outlier (-1)
    o = oracle.clue2d([0.0, 0.3, 9.0], [0.0, 0.0, 0.0], [0, 0, 0], [5.0, 1.0, 0.1], 1.0, 1.0, 2.0)
    assert o["clusterIndex"].tolist() == [0, 0, -1]
    # layers never interact
    o = oracle.clue2d([0.0, 0.0], [0.0, 0.0], [0, 1], [1.0, 1.0], 1.0, 0.5, 2.0)
    assert o["isSeed"].tolist() == [1, 1] and o["clusterIndex"].tolist() == [0, 1]


_KA = None


def _known_answer_cases():
    global _KA
    if _KA is None:
        import inspect

        import test_known_answers_gpu as ka  # the micro cases, written against a `run` callable
        _KA = {n: getattr(ka, n) for n in dir(ka)
               if n.startswith("test_") and list(inspect.signature(getattr(ka, n)).parameters) == ["run"]}
    return _KA


@needs_ref
@pytest.mark.parametrize("name", sorted(_known_answer_cases()))
def test_known_answer_micro_cases_on_the_reference(name):
    """The hand-derived micro cases (exact <= / > boundaries, ties, first-wins
    order) run through the reference's own makeClusters; the oracle must
    agree with it bit for bit on each."""
    def run(x, y, layer, w, dc, rhoc, odf):
        x, y = np.asarray(x, np.float32), np.asarray(y, np.float32)
        layer, w = np.asarray(layer, np.int32), np.asarray(w, np.float32)
        ref = oracle.ref_clue2d(x, y, layer, w, dc, rhoc, odf)
        assert_bitexact(oracle.clue2d(x, y, layer, w, dc, rhoc, odf), ref, label=name)
        return ref
    _known_answer_cases()[name](run)


@needs_ref
def test_oracle_non_finite_coordinates_on_the_reference():
    """NaN and -inf coordinates (no distance to anything, not even to the
    point itself: rho 0, an outlier) and far-away finite ones, against the
    reference's own makeClusters.  (+inf is left out: the float-to-int bin
    conversion of the reference is undefined there, and x86 and aarch64 differ.)"""
    ev = S.toy_event(5, blobs_per_layer=4, noise_per_layer=30)
    rng = np.random.default_rng(3)
    n = ev["x"].size
    k = rng.choice(n, 60, replace=False)
    ev["x"][k[:20]] = np.nan
    ev["y"][k[20:35]] = np.nan
    ev["x"][k[35:45]] = -np.inf
    ev["y"][k[45:60]] = np.float32(3e9) * np.where(rng.random(15) < 0.5, -1, 1)
    for prm in ((1.3, 2.0, 2.0), (20.0, 25.0, 2.0)):
        want = oracle.ref_clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *prm)
        got = oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *prm)
        assert_bitexact(got, want, label=str(prm))
        assert np.all(got["clusterIndex"][k[:45]] == -1)


def test_oracle_rejects_bad_layer():
    with pytest.raises(ValueError):
        oracle.clue2d([0.0], [0.0], [100], [1.0], 1.3, 2.0, 2.0)


def test_oracle_empty_events():
    """Empty events anywhere in a batch, and an empty single event."""
    b = S.uneven_batch(3, seed=16, lo=2000, hi=5000)
    o1, o2, o3 = b["offsets"][1:]
    off = np.array([0, 0, o1, o1, o2, o3, o3], np.int64)
    got = oracle.clue2d_batch(off, b["x"], b["y"], b["layer"], b["weight"], 1.3, 2.0, 2.0, n_threads=4)
    want = oracle.clue2d_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], 1.3, 2.0, 2.0)
    assert_bitexact(got, want)
    e = oracle.clue2d(np.zeros(0, np.float32), np.zeros(0, np.float32), np.zeros(0, np.int32),
                      np.zeros(0, np.float32), 1.3, 2.0, 2.0)
    assert all(v.size == 0 for v in e.values())


def test_oracle_batch_threads_match_single():
    b = S.uneven_batch(6, seed=3, lo=2000, hi=20000)
    one = oracle.clue2d_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], 1.3, 2.0, 2.0, n_threads=1)
    many = oracle.clue2d_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], 1.3, 2.0, 2.0, n_threads=4)
    assert_bitexact(many, one)
    e = 2
    ev = S.event_of(b, e)
    s, t = b["offsets"][e], b["offsets"][e + 1]
    single = oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], 1.3, 2.0, 2.0)
    assert_bitexact({k: v[s:t] for k, v in one.items()}, single)
