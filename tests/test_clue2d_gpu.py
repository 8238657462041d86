"""Parity of the CUDA CLUE 2D path with the reference, through the C ABI.

Every comparison is bit-exact on all five outputs (rho, delta,
nearestHigher, isSeed, clusterIndex): the kernels sum rho in the reference's
order with IEEE single-precision operations, so no tolerance is needed."""
import numpy as np
import pytest

import clue_gb300 as C
import oracle
from clue_gb300 import synthetic as S

from _util import assert_bitexact, golden_2d, load_golden_2d

pytestmark = pytest.mark.gpu

PRM = (1.3, 2.0, 2.0)


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


@pytest.fixture(scope="module")
def algo(cuda_lib):
    a = C.Clusterizer(*PRM, budget_bytes=48 << 30)
    yield a
    a.close()


def _oracle_batch(b, prm=PRM):
    return oracle.clue2d_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], *prm, n_threads=8)


@pytest.mark.parametrize("path", golden_2d(), ids=lambda p: p.split("/")[-1])
def test_golden_vectors(algo, path):
    ev, prm, want = load_golden_2d(path)
    algo.set_params(*prm)
    try:
        got = algo.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
    finally:
        algo.set_params(*PRM)
    assert_bitexact(got, want, label=path)


def test_toy_event_vs_oracle(algo):
    ev = S.toy_event(12345)
    got = algo.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
    assert_bitexact(got, oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *PRM))


@pytest.mark.parametrize("shuffle", [False, True])
def test_hgcal_event_vs_oracle(algo, shuffle):
    ev = S.hgcal_event(1000, shuffle=shuffle)
    got = algo.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
    assert_bitexact(got, oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *PRM))


@pytest.mark.parametrize("prm", [(20.0, 25.0, 2.0), (3.0, 4.0, 1.5), (0.5, 0.5, 5.0), (1.3, 2.0, 0.5)])
def test_parameter_sets(algo, prm):
    ev = S.toy_event(99)
    algo.set_params(*prm)
    try:
        got = algo.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
    finally:
        algo.set_params(*PRM)
    assert_bitexact(got, oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *prm), label=str(prm))


@pytest.mark.parametrize("flags", [C.HOST_MEMORY, C.HOST_MEMORY | C.NO_GRAPH, C.HOST_MEMORY | C.PLAIN])
def test_uneven_batch_host_memory(algo, flags):
    b = S.uneven_batch(24, seed=11, lo=2000, hi=60000)
    got = algo.run_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], flags=flags)
    assert_bitexact(got, _oracle_batch(b))


def test_shuffled_batch(algo):
    b = S.uneven_batch(12, seed=12, lo=2000, hi=40000, shuffle=True)
    got = algo.run_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"])
    assert_bitexact(got, _oracle_batch(b))


def _to_dev(torch, b):
    return {k: torch.from_numpy(b[k]).cuda() for k in ("x", "y", "layer", "weight")}


def _dev_out(torch, n):
    return dict(rho=torch.empty(n, dtype=torch.float32, device="cuda"),
                delta=torch.empty(n, dtype=torch.float32, device="cuda"),
                nearestHigher=torch.empty(n, dtype=torch.int32, device="cuda"),
                isSeed=torch.empty(n, dtype=torch.int32, device="cuda"),
                clusterIndex=torch.empty(n, dtype=torch.int32, device="cuda"))


@pytest.mark.parametrize("extra", [0, C.NO_GRAPH, C.PLAIN])
def test_device_memory_batch(algo, torch_cuda, extra):
    torch = torch_cuda
    b = S.uneven_batch(16, seed=13, lo=3000, hi=80000)
    d = _to_dev(torch, b)
    n = int(b["offsets"][-1])
    out = _dev_out(torch, n)
    algo.run_batch(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], out=out, flags=C.DEVICE_MEMORY | extra)
    algo.synchronize()
    got = {k: v.cpu().numpy() for k, v in out.items()}
    assert_bitexact(got, _oracle_batch(b))


def test_graph_follows_new_event_boundaries(algo, torch_cuda):
    """Same buffers, same event and point counts, other event boundaries (so
    another number of chunks): the captured graph must not be replayed."""
    torch = torch_cuda
    b = S.uneven_batch(8, seed=17, lo=3000, hi=40000)
    d = _to_dev(torch, b)
    n = int(b["offsets"][-1])
    out = _dev_out(torch, n)
    off2 = b["offsets"].copy()
    off2[1:-1] = np.sort(np.random.default_rng(3).choice(np.arange(1, n), off2.size - 2, replace=False))
    for off in (b["offsets"], off2, b["offsets"]):
        algo.run_batch(off, d["x"], d["y"], d["layer"], d["weight"], out=out, flags=C.DEVICE_MEMORY)
        algo.synchronize()
        got = {k: v.cpu().numpy() for k, v in out.items()}
        want = oracle.clue2d_batch(off, b["x"], b["y"], b["layer"], b["weight"], *PRM, n_threads=8)
        assert_bitexact(got, want)


def test_graph_replay_is_stable(algo):
    """The captured graph replays the same work: three calls, same outputs."""
    import torch
    b = S.uneven_batch(8, seed=14, lo=3000, hi=30000)
    pin = {k: torch.from_numpy(b[k]).pin_memory() for k in ("x", "y", "layer", "weight")}
    n = int(b["offsets"][-1])
    outs = []
    o = {k: torch.empty(n, dtype=torch.float32 if k in ("rho", "delta") else torch.int32).pin_memory()
         for k in ("rho", "delta", "nearestHigher", "isSeed", "clusterIndex")}
    for _ in range(3):
        for v in o.values():
            v.zero_()
        algo.run_batch(b["offsets"], pin["x"], pin["y"], pin["layer"], pin["weight"], out=o)
        outs.append({k: v.numpy().copy() for k, v in o.items()})
    want = _oracle_batch(b)
    for o in outs:
        assert_bitexact(o, want)


@pytest.mark.parametrize("cap,big_threads,big_cap", [(256, 0, 0), (256, 512, 1024), (1024, 256, 2048)])
def test_spill_and_two_class_paths_match(algo, cap, big_threads, big_cap):
    """Layers above the first pass's capacity go to the large-layer pass, and
    layers above that pass's capacity (or all of them with no second pass)
    through HBM scratch."""
    ev = S.hgcal_event(1002)
    t = algo.get_tuning()
    try:
        algo.set_tuning(layer_capacity=cap, big_threads=big_threads, big_capacity=max(big_cap, 64))
        got = algo.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
    finally:
        algo.set_tuning(**t)
    assert_bitexact(got, oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *PRM))


@pytest.mark.parametrize("threads,cap", [(256, 1024), (512, 3072), (1024, 4096), (512, 6144), (256, 2048)])
def test_tunings_give_identical_results(algo, threads, cap):
    b = S.uneven_batch(6, seed=15, lo=5000, hi=200000)
    t = algo.get_tuning()
    try:
        algo.set_tuning(threads=threads, layer_capacity=cap)
        got = algo.run_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"])
    finally:
        algo.set_tuning(**t)
    assert_bitexact(got, _oracle_batch(b))


def test_one_dense_layer(algo):
    """A single crowded layer (far above capacity, deep tiles)."""
    rng = np.random.default_rng(5)
    n = 20000
    x = rng.normal(0, 3.0, n).astype(np.float32)
    y = rng.normal(0, 3.0, n).astype(np.float32)
    layer = np.full(n, 42, np.int32)
    w = rng.exponential(1.0, n).astype(np.float32)
    got = algo.make_clusters(x, y, layer, w)
    assert_bitexact(got, oracle.clue2d(x, y, layer, w, *PRM))


def test_edge_shapes(algo):
    # empty event
    o = algo.make_clusters(np.zeros(0, np.float32), np.zeros(0, np.float32), np.zeros(0, np.int32),
                           np.zeros(0, np.float32))
    assert o["rho"].size == 0
    # single point on layer 99, far outside the grid
    o = algo.make_clusters([1e6], [-1e6], [99], [2.0])
    want = oracle.clue2d([1e6], [-1e6], [99], [2.0], *PRM)
    assert_bitexact(o, want)
    # batch with empty events in between
    b = S.uneven_batch(3, seed=16, lo=2000, hi=5000)
    off = np.array([0, 0, b["offsets"][1], b["offsets"][1], b["offsets"][2], b["offsets"][3], b["offsets"][3]],
                   np.int64)
    got = algo.run_batch(off, b["x"], b["y"], b["layer"], b["weight"])
    assert_bitexact(got, oracle.clue2d_batch(off, b["x"], b["y"], b["layer"], b["weight"], *PRM))


def test_bad_layer_is_einval(algo):
    ev = S.toy_event(1)
    layer = ev["layer"].copy()
    layer[123] = 100
    with pytest.raises(C.ClueError) as ei:
        algo.make_clusters(ev["x"], ev["y"], layer, ev["weight"])
    assert ei.value.code == C.CLUE_EINVAL
    # the handle stays usable
    got = algo.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
    assert_bitexact(got, oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *PRM))


def test_budget_is_enforced(cuda_lib):
    small = C.Clusterizer(*PRM, budget_bytes=1 << 20)
    ev = S.toy_event(2)
    with pytest.raises(C.ClueError) as ei:
        small.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
    assert ei.value.code == C.CLUE_ENOMEM
    small.close()


def test_full_size_batch_properties(algo, torch_cuda):
    """The 4096-event workload at full size: batched == plain bit for bit,
    a sample of events equals the oracle, and the label invariants hold."""
    torch = torch_cuda
    b = S.uneven_batch(4096)
    n = int(b["offsets"][-1])
    d = _to_dev(torch, b)
    out = _dev_out(torch, n)
    algo.run_batch(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], out=out, flags=C.DEVICE_MEMORY)
    algo.synchronize()
    got = {k: v.cpu().numpy() for k, v in out.items()}
    out2 = _dev_out(torch, n)
    algo.run_batch(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], out=out2,
                   flags=C.DEVICE_MEMORY | C.PLAIN)
    algo.synchronize()
    assert_bitexact({k: v.cpu().numpy() for k, v in out2.items()}, got, label="plain vs batched")
    del d, out, out2
    # invariants: seeds own their cluster id; a follower shares its nearest higher's label
    off = b["offsets"]
    for e in (0, 1, 2047, 4095):
        s, t = off[e], off[e + 1]
        ci, seed, nh = got["clusterIndex"][s:t], got["isSeed"][s:t], got["nearestHigher"][s:t]
        ids = ci[seed == 1]
        assert np.array_equal(ids, np.arange(ids.size))
        fol = (seed == 0) & (ci >= 0)
        assert np.array_equal(ci[fol], ci[nh[fol]])
    # sampled events against the oracle
    rng = np.random.default_rng(0)
    for e in rng.choice(4096, 6, replace=False):
        s, t = off[e], off[e + 1]
        ev = S.event_of(b, e)
        want = oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *PRM)
        assert_bitexact({k: v[s:t] for k, v in got.items()}, want, label=f"event {e}")


def test_host_memory_pipelined_large_batch(algo):
    """Host-memory batches of at least 16M points run as overlapped
    sub-batches (H2D, kernels and D2H on three streams over two device slots):
    bit-identical to the single H2D-kernels-D2H sequence and, on sampled
    events, to the oracle."""
    b = S.uneven_batch(760, seed=29, lo=30000, hi=70000)
    n = int(b["offsets"][-1])
    assert n >= 32 << 20  # four or more sub-batches
    got = algo.run_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"])
    st = algo.last_run_stats()
    nchunks = int(np.sum((np.diff(b["offsets"]) + 4095) // 4096))  # event-aligned chunks of 4096 points
    assert 16 * n + 4 * nchunks < st["h2d_bytes"] < 16 * n + 4 * nchunks + 64 * b["offsets"].size
    assert 20 * n < st["d2h_bytes"] < 20 * n + 4096  # outputs plus one status block per sub-batch
    assert st["kernel_launches"] >= 8 * 4  # four or more sub-batches of 8 kernels or more
    ref = algo.run_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], flags=C.NO_PIPELINE)
    st = algo.last_run_stats()
    assert (st["h2d_bytes"], st["d2h_bytes"]) == (16 * n + 12 * b["offsets"].size + 4 * nchunks, 20 * n + 32)
    assert_bitexact(got, ref)
    for e in (0, 359, 759):
        s, t = b["offsets"][e], b["offsets"][e + 1]
        want = oracle.clue2d(b["x"][s:t], b["y"][s:t], b["layer"][s:t], b["weight"][s:t], *PRM)
        assert_bitexact({k: v[s:t] for k, v in got.items()}, want, label=f"event {e}")
    # an invalid layer in a late sub-batch is reported, and the handle recovers
    bad = b["layer"].copy()
    bad[n - 5] = 100
    with pytest.raises(C.ClueError, match="layer"):
        algo.run_batch(b["offsets"], b["x"], b["y"], bad, b["weight"])
    again = algo.run_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"])
    assert_bitexact(again, ref)


def test_layer_order_rule_and_run_stats(cuda_lib):
    """Batches with a few layers per CTA take their layers largest first (one
    more kernel); a single event keeps the event order and runs one pass.  The order only
    changes which CTA runs which layer: results are identical to the
    one-event-per-launch form, and the run statistics count what was queued."""
    algo = C.Clusterizer(*PRM)  # default tuning: several CTAs per SM, so 200 events are a few layers per CTA
    b = S.uneven_batch(200, seed=41, lo=5000, hi=60000)
    n = int(b["offsets"][-1])
    got = algo.run_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], flags=C.NO_PIPELINE)
    ordered = algo.last_run_stats()
    nchunks = int(np.sum((np.diff(b["offsets"]) + 4095) // 4096))
    assert ordered["h2d_bytes"] == 16 * n + 12 * b["offsets"].size + 4 * nchunks
    ev = S.event_of(b, 7)
    algo.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
    single = algo.last_run_stats()
    assert single["kernel_launches"] == 8  # a single event runs one wide pass per layer
    t = algo.get_tuning()
    two_class = t["big_threads"] > 0 and t["big_capacity"] > t["layer_capacity"]
    assert ordered["kernel_launches"] == 8 + 1 + (1 if two_class else 0)  # + the size order (+ the large-layer pass)
    ref = algo.run_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], flags=C.PLAIN)
    assert algo.last_run_stats()["kernel_launches"] == 200 * single["kernel_launches"]
    algo.close()
    assert_bitexact(got, ref)


def test_graph_only_for_repeated_shapes(cuda_lib):
    """A new shape runs by direct launches, a shape seen twice in a row is
    captured, then replayed; another shape re-captures.  Every mode gives the
    same outputs and reports the same kernel count."""
    import torch
    algo = C.Clusterizer(*PRM)
    bs = [S.uneven_batch(6, seed=s, lo=3000, hi=20000) for s in (61, 62)]
    dev = [{k: torch.from_numpy(b[k]).cuda() for k in ("x", "y", "layer", "weight")} for b in bs]
    outs = [{k: torch.empty(int(b["offsets"][-1]), dtype=torch.float32 if k in ("rho", "delta") else torch.int32,
                            device="cuda") for k in ("rho", "delta", "nearestHigher", "isSeed", "clusterIndex")}
            for b in bs]
    counts = []
    for i in (0, 1, 0, 0, 0, 1, 1, 1):  # direct, direct, direct, capture, replay, direct, capture, replay
        for v in outs[i].values():
            v.zero_()
        torch.cuda.synchronize()  # the handle runs on its own stream: the fill must be done first
        algo.run_batch(bs[i]["offsets"], dev[i]["x"], dev[i]["y"], dev[i]["layer"], dev[i]["weight"], out=outs[i],
                       flags=C.DEVICE_MEMORY)
        algo.synchronize()
        counts.append(algo.last_run_stats()["kernel_launches"])
        assert_bitexact({k: v.cpu().numpy() for k, v in outs[i].items()}, _oracle_batch(bs[i]))
    assert counts[2:5] == [counts[0]] * 3 and counts[5:] == [counts[1]] * 3
    algo.close()
