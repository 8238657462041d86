"""The serving loop: continuous batching with overlapping in-flight batches.

The key property: every request's result is bit-identical whether the event
runs alone (clue_run_event) or inside whatever batch the server formed."""
import threading
import time

import numpy as np
import pytest

import clue_gb300 as C
import oracle
from clue_gb300 import synthetic as S

from _util import assert_bitexact

pytestmark = pytest.mark.gpu

PRM = (1.3, 2.0, 2.0)


@pytest.fixture(scope="module")
def events():
    b = S.uneven_batch(48, seed=21, lo=2000, hi=120000)
    return [S.event_of(b, e) for e in range(48)]


@pytest.fixture(scope="module")
def alone(events, cuda_lib):
    a = C.Clusterizer(*PRM)
    outs = [a.make_clusters(e["x"], e["y"], e["layer"], e["weight"]) for e in events]
    a.close()
    return outs


def test_results_identical_alone_and_in_the_mix(events, alone):
    srv = C.Server(*PRM, budget_bytes=8 << 30, max_inflight=2, max_batch_events=6)
    rng = np.random.default_rng(3)
    ids = [None] * len(events)
    outs = [None] * len(events)

    def client(k0):
        for k in range(k0, len(events), 3):
            time.sleep(float(rng.exponential(0.002)))
            ids[k], outs[k] = srv.submit(**events[k])

    th = [threading.Thread(target=client, args=(i,)) for i in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    lats = []
    for k, rid in enumerate(ids):
        st, lat = srv.poll(rid, timeout_ms=60000)
        assert st == C.CLUE_OK
        lats.append(lat)
        assert_bitexact(outs[k], alone[k], label=f"request {k}")
    stats = srv.stats()
    assert stats["completed"] == len(events)
    # how many batches form depends on arrival timing; batching itself is
    # asserted under a burst in test_burst_overlaps_batches_on_device
    assert stats["batches"] <= len(events)
    assert all(l > 0 for l in lats)
    assert stats["p99_ms"] >= stats["p50_ms"] > 0
    srv.close()


def test_burst_overlaps_batches_on_device(events, alone):
    srv = C.Server(*PRM, budget_bytes=8 << 30, max_inflight=2, max_batch_events=4)
    # one bulk submit: the scheduler sees the whole burst at once
    off = np.concatenate([[0], np.cumsum([e["x"].size for e in events])]).astype(np.int64)
    cat = {k: np.concatenate([e[k] for e in events]) for k in ("x", "y", "layer", "weight")}
    reqs = srv.submit_many(off, cat["x"], cat["y"], cat["layer"], cat["weight"])
    srv.drain(timeout_ms=60000)
    for k, (rid, out) in enumerate(reqs):
        st, _ = srv.poll(rid, timeout_ms=0)
        assert st == C.CLUE_OK
        assert_bitexact(out, alone[k])
    st = srv.stats()
    assert st["max_inflight_seen"] >= 2, st
    assert st["mean_batch_events"] > 1
    srv.close()


def test_one_request_against_the_oracle(events):
    srv = C.Server(*PRM, budget_bytes=4 << 30, max_inflight=1, max_batch_events=8)
    e = events[5]
    rid, out = srv.submit(**e)
    assert srv.poll(rid, timeout_ms=60000)[0] == C.CLUE_OK
    assert_bitexact(out, oracle.clue2d(e["x"], e["y"], e["layer"], e["weight"], *PRM))
    srv.close()


def _uniform_event(n, seed):
    rng = np.random.default_rng(seed)
    return dict(x=rng.uniform(-240, 240, n).astype(np.float32), y=rng.uniform(-240, 240, n).astype(np.float32),
                layer=rng.integers(0, 100, n).astype(np.int32), weight=rng.exponential(1.0, n).astype(np.float32))


def test_admission_rejects_an_event_larger_than_the_budget_admits():
    """slot_capacity_points is the largest event that fits the budget while
    the other slot holds its start-up buffers; one point more is refused."""
    srv = C.Server(*PRM, budget_bytes=96 << 20, max_inflight=2, max_batch_events=4)
    cap = srv.stats()["slot_capacity_points"]
    assert cap > 1000
    with pytest.raises(C.ClueError) as ei:
        srv.submit(**_uniform_event(cap + 1, 1))
    assert ei.value.code == C.CLUE_ENOMEM
    small = _uniform_event(cap // 2, 2)
    rid, out = srv.submit(**small)  # half a slot still fits
    assert srv.poll(rid, timeout_ms=60000)[0] == C.CLUE_OK
    assert_bitexact(out, oracle.clue2d(small["x"], small["y"], small["layer"], small["weight"], *PRM))
    srv.close()


def test_large_events_share_the_budget_and_wait_for_memory():
    """Two events each larger than half the budget's share: the first takes
    what the idle slot leaves of the budget, the second waits at the head of
    the queue until the first batch has finished (its slot then gives its
    memory back), instead of being refused.  Both results are bit-identical
    to the oracle, as is a small event queued behind them."""
    budget = 96 << 20
    srv = C.Server(*PRM, budget_bytes=budget, max_inflight=2, max_batch_events=4)
    cap = srv.stats()["slot_capacity_points"]
    # each above what an equal split of the budget would admit, and two of
    # them together above the budget (memory_waits below shows the wait)
    big = int(cap * 0.7)
    evs = [_uniform_event(big, 11), _uniform_event(big, 12), _uniform_event(5000, 13)]
    off = np.array([0, big, 2 * big, 2 * big + 5000], np.int64)
    cat = {k: np.concatenate([e[k] for e in evs]) for k in ("x", "y", "layer", "weight")}
    reqs = srv.submit_many(off, cat["x"], cat["y"], cat["layer"], cat["weight"])
    srv.drain(timeout_ms=120000)
    for (rid, out), e in zip(reqs, evs):
        assert srv.poll(rid, timeout_ms=0)[0] == C.CLUE_OK
        assert_bitexact(out, oracle.clue2d(e["x"], e["y"], e["layer"], e["weight"], *PRM))
    st = srv.stats()
    assert st["memory_waits"] >= 1, st
    assert st["completed"] == 3
    srv.close()
