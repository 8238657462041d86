"""clue_run_event_noalloc: the allocation-free entry point.

It exists for callers that cannot call cudaMalloc themselves -- for example
a host framework that hands the whole device to its own memory pool, or
real-time code that must not touch the allocator after start-up.  It keeps
its scratch in a fixed array compiled into the library, so it must give
exactly what the oracle and the regular entry point give, call after call,
even though every call reuses the same scratch.  The comparison is bit for
bit (the project's tolerance for CLUE outputs is zero).

Cases: the warm-up call (n = 0, no data), two different events back to back
against the oracle and the regular entry point, a single layer far above the
on-chip capacity (the spill area inside the fixed scratch), an event at the
262,144-point limit with most points on one layer (the whole scratch layout
in use), an invalid layer followed by a correct call, no change in the
device's free memory across a call, and the size limit.

This file is collected last so that, in a run that stops at the first
failure, every other test has already run; it also passes on its own.
"""
import ctypes

import numpy as np
import pytest

import clue_gb300 as C
import oracle
from clue_gb300 import synthetic as S

from _util import assert_bitexact

pytestmark = pytest.mark.gpu

PRM = (1.3, 2.0, 2.0)
KEYS = ("rho", "delta", "nearestHigher", "isSeed", "clusterIndex")
LIMIT = 1 << 18


def _call(torch, dev, stream, out=None):
    n = dev["x"].numel()
    if out is None:
        out = {k: torch.full((n,), -7, dtype=torch.float32 if k in ("rho", "delta") else torch.int32, device="cuda")
               for k in KEYS}
    o = C.outputs_struct(out)
    torch.cuda.synchronize()  # the fill above ran on torch's stream, the call runs on `stream`
    rc = C.lib().clue_run_event_noalloc(ctypes.byref(C.Params(*PRM)), n, dev["x"].data_ptr(), dev["y"].data_ptr(),
                                        dev["layer"].data_ptr(), dev["weight"].data_ptr(), ctypes.byref(o),
                                        stream.cuda_stream)
    return rc, out


def _dev(torch, ev):
    return {k: torch.from_numpy(np.ascontiguousarray(ev[k])).cuda() for k in ("x", "y", "layer", "weight")}


def _noalloc(torch, ev, stream):
    rc, out = _call(torch, _dev(torch, ev), stream)
    C.check(rc)
    return {k: v.cpu().numpy() for k, v in out.items()}


def _oracle(ev):
    return oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *PRM)


def _one_dense_layer(seed, n, layer=7, other=0):
    """``n`` points: Gaussian blobs (sigma 1 cm, about 60 points each) spread
    over the grid in one layer, plus ``other`` noise points on other layers."""
    rng = np.random.default_rng(seed)
    m = n - other
    nb = max(1, m // 60)
    cx, cy = rng.uniform(-240, 240, nb), rng.uniform(-240, 240, nb)
    blob = rng.integers(0, nb, m)
    x = (cx[blob] + rng.standard_normal(m)).astype(np.float32)
    y = (cy[blob] + rng.standard_normal(m)).astype(np.float32)
    lay = np.full(m, layer, np.int32)
    if other:
        x = np.concatenate([x, rng.uniform(-250, 250, other).astype(np.float32)])
        y = np.concatenate([y, rng.uniform(-250, 250, other).astype(np.float32)])
        lay = np.concatenate([lay, rng.choice(np.setdiff1d(np.arange(100), [layer]), other).astype(np.int32)])
    w = np.exp(0.5 * rng.standard_normal(n)).astype(np.float32)
    return dict(x=x, y=y, layer=lay, weight=w)


def test_noalloc_warm_up_call_needs_no_data():
    """n = 0 with every pointer NULL: the start-up call that creates the
    scratch array and loads the kernels, and nothing else."""
    assert C.lib().clue_run_event_noalloc(None, 0, None, None, None, None, None, None) == C.CLUE_OK
    assert C.lib().clue_run_event_noalloc(None, 0, None, None, None, None, None, None) == C.CLUE_OK


def test_noalloc_matches_the_oracle_and_the_regular_entry_point_twice_in_a_row():
    import torch
    assert torch.cuda.is_available()
    stream = torch.cuda.Stream()
    regular = C.Clusterizer(*PRM)
    # two different events back to back: the second must not see the first's leftovers
    events = [S.toy_event(31), S.event_of(S.uneven_batch(3, seed=41, lo=60000, hi=150000), 2)]
    for ev in events:
        got = _noalloc(torch, ev, stream)
        assert_bitexact(got, _oracle(ev), KEYS, label=f"{ev['x'].size} points vs oracle")
        want = regular.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
        assert_bitexact(got, want, KEYS, label=f"{ev['x'].size} points vs regular entry point")
    regular.close()


def test_noalloc_single_layer_above_on_chip_capacity():
    """20,000 points in one layer: far above the 4,096 points a layer kernel
    holds on chip, so the layer runs from the spill area of the fixed scratch."""
    import torch
    ev = _one_dense_layer(5, 20000)
    got = _noalloc(torch, ev, torch.cuda.Stream())
    assert_bitexact(got, _oracle(ev), KEYS, label="20,000 points in one layer")


def test_noalloc_at_the_point_limit_with_one_dense_layer():
    """262,144 points, 250,000 of them in one layer: every part of the fixed
    layout (grouped copies, spill records, per-CTA tile tables) is in use."""
    import torch
    ev = _one_dense_layer(6, LIMIT, other=LIMIT - 250000)
    assert ev["x"].size == LIMIT
    stream = torch.cuda.Stream()
    want = _oracle(ev)
    for rep in range(2):
        got = _noalloc(torch, ev, stream)
        assert_bitexact(got, want, KEYS, label=f"262,144 points, call {rep}")


def test_noalloc_invalid_layer_then_a_correct_call():
    import torch
    stream = torch.cuda.Stream()
    ev = S.toy_event(8)
    bad = dict(ev)
    bad["layer"] = ev["layer"].copy()
    bad["layer"][4321] = 100
    rc, _ = _call(torch, _dev(torch, bad), stream)
    assert rc == C.CLUE_EINVAL
    assert "layer" in C.last_error()
    got = _noalloc(torch, ev, stream)  # the status word was cleared: the next call is clean
    assert_bitexact(got, _oracle(ev), KEYS, label="after an invalid layer")


def test_noalloc_device_memory_unchanged_across_a_call():
    """After the warm-up and a first call, a further call leaves the device's
    free memory exactly as it was: nothing is allocated per call."""
    import torch
    stream = torch.cuda.Stream()
    assert C.lib().clue_run_event_noalloc(None, 0, None, None, None, None, None, None) == C.CLUE_OK
    ev = S.event_of(S.uneven_batch(2, seed=77, lo=80000, hi=120000), 1)
    dev = _dev(torch, ev)
    rc, out = _call(torch, dev, stream)
    C.check(rc)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc, out = _call(torch, dev, stream, out)
    C.check(rc)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert_bitexact({k: v.cpu().numpy() for k, v in out.items()}, _oracle(ev), KEYS)


def test_noalloc_rejects_events_above_its_limit():
    import torch
    n = LIMIT + 1
    z = torch.zeros(n, dtype=torch.float32, device="cuda")
    zi = torch.zeros(n, dtype=torch.int32, device="cuda")
    o = C.Outputs(z.data_ptr(), z.data_ptr(), zi.data_ptr(), zi.data_ptr(), zi.data_ptr())
    rc = C.lib().clue_run_event_noalloc(ctypes.byref(C.Params(*PRM)), n, z.data_ptr(), z.data_ptr(),
                                        zi.data_ptr(), z.data_ptr(), ctypes.byref(o), None)
    assert rc == C.CLUE_EINVAL
    assert "262144" in C.last_error()
