"""Parity of the CUDA CLUE3D path with the reference tracksterizer through
the C ABI: bit-exact on rho, delta (transverse, layers), nearestHigher
(layer, index), isSeed, tracksterIndex and the per-event trackster count."""
import numpy as np
import pytest

import clue_gb300 as C
import oracle
from clue_gb300 import synthetic as S

from _util import KEYS_3D, assert_bitexact, golden_3d, load_golden_3d, assert_bitexact_nan

pytestmark = pytest.mark.gpu

GPU2ORACLE = dict(rho="rho", delta_transverse="delta_t", delta_layers="delta_l", nh_layer="nh_layer",
                  nh_index="nh_idx", isSeed="isSeed", tracksterIndex="tracksterIndex")
CONFIG4 = dict(n_layers=100, density_sibling_layers=2, nh_sibling_layers=2, critical_density=0.5)


@pytest.fixture(scope="module")
def algo(cuda_lib):
    a = C.Clusterizer(1.3, 2.0, 2.0, budget_bytes=32 << 30)
    yield a
    a.close()


def _as_oracle(out, s=None, t=None):
    return {GPU2ORACLE[k]: (v[s:t] if s is not None else v) for k, v in out.items()}


def _oracle_batch(b, prm):
    outs, nts = [], []
    for e in range(b["offsets"].size - 1):
        o, nt = oracle.clue3d(S.event3d_of(b, e), **prm)
        outs.append(o)
        nts.append(nt)
    return {k: np.concatenate([o[k] for o in outs]) for k in KEYS_3D}, np.array(nts)


@pytest.mark.parametrize("path", golden_3d(), ids=lambda p: p.split("/")[-1])
def test_golden_vectors_3d(algo, path):
    ev, prm, want, nt = load_golden_3d(path)
    off = np.array([0, ev["z"].size], np.int64)
    out, nts = algo.run_clue3d(off, ev, params=prm)
    assert int(nts[0]) == nt
    assert_bitexact(_as_oracle(out), want, KEYS_3D, label=path)


@pytest.mark.parametrize("prm", [{}, CONFIG4, dict(n_layers=100, density_on_same_layer=1, nh_on_same_layer=1)])
def test_batch_vs_oracle(algo, prm):
    nl = prm.get("n_layers", 94)
    b = S.clue3d_batch(8, seed0=300, n_layers=nl)
    out, nts = algo.run_clue3d(b["offsets"], b, params=prm)
    want, wnt = _oracle_batch(b, prm)
    assert np.array_equal(nts, wnt)
    assert_bitexact(_as_oracle(out), want, KEYS_3D)


def test_device_memory_and_scintillator(algo):
    import torch
    b = S.clue3d_batch(5, seed0=400, n_layers=100)
    rng = np.random.default_rng(1)
    n = b["z"].size
    b["isSilicon"] = (rng.random(n) < 0.5).astype(np.int32)
    b["radius"] = rng.uniform(0.5, 3.0, n).astype(np.float32)
    b["phi"][::7] = np.float32(np.pi)          # wrap edge: phi bin 126 lands in the next eta row
    b["phi"][3::7] = -np.float32(np.pi)
    b["eta"][::11] = np.float32(3.0)
    dev = {k: torch.from_numpy(np.ascontiguousarray(b[k])).cuda()
           for k in ("z", "eta", "phi", "r_over_absz", "radius", "layer", "energy", "isSilicon")}
    out = {k: torch.empty(n, dtype=torch.float32 if k in ("rho", "delta_transverse") else torch.int32,
                          device="cuda") for k in GPU2ORACLE}
    algo.run_clue3d(b["offsets"], dev, params=dict(n_layers=100), flags=C.DEVICE_MEMORY, out=out)
    algo.synchronize()
    got = {k: v.cpu().numpy() for k, v in out.items()}
    want, _ = _oracle_batch(b, dict(n_layers=100))
    assert_bitexact(_as_oracle(got), want, KEYS_3D)


def test_bad_layer_3d(algo):
    ev = S.clue3d_event(9, n_clusters=500, n_layers=94)
    ev["layer"][10] = 94
    with pytest.raises(C.ClueError) as ei:
        algo.run_clue3d(np.array([0, 500], np.int64), ev)
    assert ei.value.code == C.CLUE_EINVAL
    ev["layer"][10] = 3
    out, nt = algo.run_clue3d(np.array([0, 500], np.int64), ev)
    want, wnt = oracle.clue3d(ev)
    assert nt[0] == wnt
    assert_bitexact(_as_oracle(out), want, KEYS_3D)


def test_non_finite_and_huge_phi_3d(algo):
    """A phi that stays far outside [-pi, pi] after the reference's range
    reduction (|phi| of 1e12 here) is rejected (the reference would index
    outside its tile); NaN and +-inf phi reduce to NaN and take phi bin 0, as
    in the oracle."""
    ev = S.clue3d_event(9, n_clusters=500, n_layers=94)
    ev["phi"][10] = np.float32(1e12)
    with pytest.raises(C.ClueError) as ei:
        algo.run_clue3d(np.array([0, 500], np.int64), ev)
    assert ei.value.code == C.CLUE_EINVAL
    ev["phi"][10] = np.nan
    ev["phi"][11] = np.inf
    ev["phi"][12] = -np.inf
    out, nt = algo.run_clue3d(np.array([0, 500], np.int64), ev)
    want, wnt = oracle.clue3d(ev)
    assert nt[0] == wnt
    assert_bitexact_nan(_as_oracle(out), want, KEYS_3D)


@pytest.mark.parametrize("prm", [{}, dict(density_sibling_layers=2, nh_sibling_layers=2, critical_density=0.5)])
def test_side_boundary_and_high_eta_3d(algo, prm):
    """Dense clusters on layers 44-51 around the detector sides' split (94
    layers: density windows stop below 47, the upper nearest-higher window
    starts at 48), eta up to 3.0, phi in a narrow band (the event the CPU
    tests pin on the reference)."""
    rng = np.random.default_rng(11)
    ev = S.clue3d_event(12, n_clusters=3000, n_layers=94, eta_range=(2.8, 3.0))
    layer = rng.integers(44, 52, ev["z"].size).astype(np.int32)
    phi = rng.uniform(0.0, 0.4, ev["z"].size).astype(np.float32)
    z = S.layer_z(94)[layer].astype(np.float32)
    r = ev["r_over_absz"] * z
    ev.update(layer=layer, phi=phi, z=z, x=(r * np.cos(phi)).astype(np.float32), y=(r * np.sin(phi)).astype(np.float32))
    n = ev["z"].size
    out, nt = algo.run_clue3d(np.array([0, n], np.int64), ev, params=dict(n_layers=94, **prm))
    want, wnt = oracle.clue3d(ev, **prm)
    assert nt[0] == wnt
    assert_bitexact(_as_oracle(out), want, KEYS_3D)
