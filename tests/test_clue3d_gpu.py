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


def _event3d(eta, phi, layer, seed):
    """A CLUE3D event from given eta, phi and layer (the other fields derived
    as the synthetic generator derives them)."""
    rng = np.random.default_rng(seed)
    k = eta.size
    z = S.layer_z(100)[layer]
    roa = (1.0 / np.sinh(eta.astype(np.float64))).astype(np.float32)
    r = roa * z
    phi = phi.astype(np.float32)
    return dict(x=(r * np.cos(phi)).astype(np.float32), y=(r * np.sin(phi)).astype(np.float32),
                z=z.astype(np.float32), eta=eta.astype(np.float32), phi=phi, r_over_absz=roa,
                radius=np.full(k, 2.0, np.float32), layer=layer.astype(np.int32),
                energy=np.exp(0.7 * rng.standard_normal(k)).astype(np.float32), isSilicon=np.ones(k, np.int32))


def test_dense_rows_and_staging_overflow_3d(algo):
    """Rows far from the typical three entries: one (layer, eta) row with an
    entry in every phi column (the column-count rank with a full mask), one
    column holding 60 entries (the walked rank and walked visits), and a slab
    of four layers with 3,000 clusters, above the searches' on-chip staging
    capacity (the global-memory path), each with a sprinkle of other clusters,
    in shuffled order; every output against the oracle."""
    rng = np.random.default_rng(2024)
    bw = 2 * np.pi / 126
    evs = []
    # every phi column of layer 10, eta bin 2, plus neighbours in eta and layer
    c = np.arange(126)
    phi = (c + rng.uniform(0.1, 0.9, 126)) * bw - np.pi
    eta = np.full(126, 1.5 + 2.5 / 20)
    lay = np.full(126, 10)
    eta = np.concatenate([eta, rng.uniform(1.5, 1.8, 400)])
    phi = np.concatenate([phi, rng.uniform(-np.pi, np.pi, 400)])
    lay = np.concatenate([lay, rng.choice([8, 9, 11, 12], 400)])  # the full row keeps one entry per column
    evs.append((eta, phi, lay))
    # 60 clusters in one (layer, eta, phi) bin, neighbours around it
    eta = np.concatenate([np.full(60, 1.5 + 5.5 / 20), rng.uniform(1.7, 1.9, 300)])
    phi = np.concatenate([(40 + rng.uniform(0.05, 0.95, 60)) * bw - np.pi, (rng.uniform(36, 45, 300)) * bw - np.pi])
    lay = np.concatenate([np.full(60, 30), rng.integers(27, 34, 300)])
    evs.append((eta, phi, lay))
    # 3,000 clusters in layers 20-23 (plus siblings): above the staging capacity
    eta = rng.uniform(1.5, 3.0, 3600)
    phi = rng.uniform(-np.pi, np.pi, 3600)
    lay = np.concatenate([rng.integers(20, 24, 3000), rng.integers(16, 28, 600)])
    evs.append((eta, phi, lay))
    events = []
    for i, (eta, phi, lay) in enumerate(evs):
        perm = rng.permutation(eta.size)
        events.append(_event3d(eta[perm], phi[perm], lay[perm], 50 + i))
    b = S.concat3d(events)
    out, nts = algo.run_clue3d(b["offsets"], b, params=CONFIG4)
    want, wnt = _oracle_batch(b, CONFIG4)
    assert np.array_equal(nts, wnt)
    assert_bitexact(_as_oracle(out), want, KEYS_3D, label="dense rows")
