"""The autotuner: it times the work decompositions of the layer kernel on a
batch (first pass: threads and on-chip capacity; second pass: the
large-layer pass), checks that every candidate gives bit-identical outputs,
keeps the fastest and records it per GPU and workload."""
import json

import numpy as np
import pytest

import clue_gb300 as C
import oracle
from clue_gb300 import synthetic as S

from _util import assert_bitexact

pytestmark = pytest.mark.gpu

PRM = (1.3, 2.0, 2.0)


def _dev_batch(torch, b):
    n = int(b["offsets"][-1])
    d = {k: torch.from_numpy(b[k]).cuda() for k in ("x", "y", "layer", "weight")}
    out = {k: torch.empty(n, dtype=torch.float32 if k in ("rho", "delta") else torch.int32, device="cuda")
           for k in ("rho", "delta", "nearestHigher", "isSeed", "clusterIndex")}
    return d, out


def test_autotune_choice_cache_and_results(tmp_path, cuda_lib):
    import torch
    b = S.uneven_batch(24, seed=41, lo=20000, hi=200000)
    d, out = _dev_batch(torch, b)
    cache = tmp_path / "tune.jsonl"
    algo = C.Clusterizer(*PRM, budget_bytes=16 << 30)
    chosen = algo.autotune(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], out, cache_path=str(cache))
    assert chosen == algo.get_tuning()
    assert chosen["threads"] in (128, 256, 512) and chosen["work_tile_cm"] == 0.0
    assert chosen["big_threads"] == 0 or chosen["big_capacity"] > chosen["layer_capacity"]
    lines = [json.loads(l) for l in cache.read_text().splitlines()]
    assert len(lines) == 1 and lines[0]["format"] == 2
    assert (lines[0]["threads"], lines[0]["layer_capacity"], lines[0]["big_threads"], lines[0]["big_capacity"]) == \
        (chosen["threads"], chosen["layer_capacity"], chosen["big_threads"], chosen["big_capacity"])
    # the chosen decomposition gives the reference's results
    algo.run_batch(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], out=out, flags=C.DEVICE_MEMORY)
    algo.synchronize()
    want = oracle.clue2d_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], *PRM, n_threads=8)
    assert_bitexact({k: v.cpu().numpy() for k, v in out.items()}, want)
    algo.close()
    # a new handle reuses the cached choice without timing (no new cache line)
    algo2 = C.Clusterizer(*PRM, budget_bytes=16 << 30)
    again = algo2.autotune(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], out, cache_path=str(cache))
    assert again == chosen
    assert len(cache.read_text().splitlines()) == 1
    algo2.close()


def test_reserved_work_tile_is_rejected(cuda_lib):
    algo = C.Clusterizer(*PRM)
    with pytest.raises(C.ClueError, match="work_tile_cm"):
        algo.set_tuning(work_tile_cm=1.0)
    with pytest.raises(C.ClueError):
        algo.set_tuning(threads=96)
    algo.close()
