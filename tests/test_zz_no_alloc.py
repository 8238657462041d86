"""clue_run_event_noalloc: the allocation-free entry point.

It exists for callers that cannot call cudaMalloc themselves -- for example
a host framework that hands the whole device to its own memory pool, or
real-time code that must not touch the allocator after start-up.  It keeps
its scratch in a fixed array compiled into the library, so it must give
exactly what the regular entry point gives, call after call, even though
every call reuses the same scratch.  The comparison is bit for bit (the
project's tolerance for CLUE outputs is zero).

This file is collected last so that, in a run that stops at the first
failure, every other test has already run; it also passes on its own.
"""
import ctypes

import numpy as np
import pytest

import clue_gb300 as C
from clue_gb300 import synthetic as S

from _util import assert_bitexact

pytestmark = pytest.mark.gpu

PRM = (1.3, 2.0, 2.0)
KEYS = ("rho", "delta", "nearestHigher", "isSeed", "clusterIndex")


def _noalloc(torch, ev, stream):
    dev = {k: torch.from_numpy(np.ascontiguousarray(ev[k])).cuda() for k in ("x", "y", "layer", "weight")}
    n = dev["x"].numel()
    out = {k: torch.full((n,), -7, dtype=torch.float32 if k in ("rho", "delta") else torch.int32, device="cuda")
           for k in KEYS}
    o = C.outputs_struct(out)
    rc = C.lib().clue_run_event_noalloc(ctypes.byref(C.Params(*PRM)), n, dev["x"].data_ptr(), dev["y"].data_ptr(),
                                        dev["layer"].data_ptr(), dev["weight"].data_ptr(), ctypes.byref(o),
                                        stream.cuda_stream)
    C.check(rc)
    return {k: v.cpu().numpy() for k, v in out.items()}


def test_noalloc_matches_the_regular_entry_point_twice_in_a_row():
    import torch
    assert torch.cuda.is_available()
    stream = torch.cuda.Stream()
    regular = C.Clusterizer(*PRM)
    # two different events back to back: the second must not see the first's leftovers
    events = [S.toy_event(31), S.event_of(S.uneven_batch(3, seed=41, lo=60000, hi=150000), 2)]
    for ev in events:
        want = regular.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
        got = _noalloc(torch, ev, stream)
        assert_bitexact(got, want, KEYS, label=f"{ev['x'].size} points")
    regular.close()


def test_noalloc_rejects_events_above_its_limit():
    import torch
    n = (1 << 18) + 1
    z = torch.zeros(n, dtype=torch.float32, device="cuda")
    zi = torch.zeros(n, dtype=torch.int32, device="cuda")
    o = C.Outputs(z.data_ptr(), z.data_ptr(), zi.data_ptr(), zi.data_ptr(), zi.data_ptr())
    rc = C.lib().clue_run_event_noalloc(ctypes.byref(C.Params(*PRM)), n, z.data_ptr(), z.data_ptr(),
                                        zi.data_ptr(), z.data_ptr(), ctypes.byref(o), None)
    assert rc == C.CLUE_EINVAL
    assert "262144" in C.last_error()
