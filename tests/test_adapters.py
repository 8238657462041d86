"""The C++ adapters with the reference producers' signatures:
include/CLUEAlgoGB300.h (CLUEAlgoSerial::makeClusters) and
include/CLUEAlgoGB300CUDA.h (CLUEAlgoCUDA::makeClusters, results resident on
the device, then the CUDA CLUEOutputProducer's transfer).  tests/adapter_demo.cc
drives both like CLUESerialClusterizer / CLUECUDAClusterizer do."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import clue_gb300 as C
import oracle
from clue_gb300 import formats as F
from clue_gb300 import synthetic as S

from _util import assert_bitexact, KEYS_2D

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
DEMO = os.path.join(ROOT, "tests", "adapter_demo.cc")


def _gxx():
    gxx = shutil.which("g++")
    if not gxx or not os.path.exists(os.path.join(CUDA, "include", "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are missing")
    return gxx


def test_adapters_compile():
    """Both adapter headers compile against the C ABI (no GPU needed)."""
    subprocess.run([_gxx(), "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(CUDA, "include"), DEMO], check=True)


def _read_dump(path, sizes):
    raw = np.fromfile(path, dtype=np.uint8)
    pos, res = 0, []
    for n in sizes:
        for _ in range(2):  # serial adapter, then device adapter
            assert int(raw[pos:pos + 4].view("<u4")[0]) == n
            pos += 4
            o = {}
            for k in KEYS_2D:
                dt = np.float32 if k in ("rho", "delta") else np.int32
                o[k] = raw[pos:pos + 4 * n].view(dt).copy()
                pos += 4 * n
            res.append(o)
    assert pos == raw.size
    return res


@pytest.mark.gpu
def test_adapters_match_oracle(tmp_path, cuda_lib):
    exe = str(tmp_path / "adapter_demo")
    libdir = os.path.dirname(C.LIB_PATH)
    subprocess.run([_gxx(), "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(CUDA, "include"), DEMO, "-o", exe, "-L", libdir, "-lclue_gb300",
                    "-Wl,-rpath," + libdir, "-L", os.path.join(CUDA, "lib64"), "-lcudart",
                    "-Wl,-rpath," + os.path.join(CUDA, "lib64")], check=True)
    b = S.uneven_batch(3, seed=21, lo=2000, hi=30000)
    evs = [S.event_of(b, e) for e in range(3)]
    empty = {k: v[:0] for k, v in evs[0].items()}
    evs.insert(1, empty)
    src = tmp_path / "raw2D.bin"
    F.write_raw2d(src, evs)
    prm = (1.3, 2.0, 2.0)
    dst = tmp_path / "dump.bin"
    subprocess.run([exe, str(src), str(dst), *map(str, prm)], check=True)
    got = _read_dump(dst, [e["x"].size for e in evs])
    for k, ev in enumerate(evs):
        want = oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *prm)
        assert_bitexact(got[2 * k], want)
        assert_bitexact(got[2 * k + 1], want)


@pytest.mark.gpu
def test_set_stream_follows_the_callers_stream(cuda_lib):
    import torch
    ev = S.toy_event(5, blobs_per_layer=5, noise_per_layer=50)
    want = oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], 20.0, 25.0, 2.0)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in ev.items()}
    algo = C.Clusterizer(20.0, 25.0, 2.0)
    n = ev["x"].size
    for s in (torch.cuda.Stream(), None, torch.cuda.Stream()):
        algo.set_stream(s.cuda_stream if s is not None else None)
        out = {k: torch.empty(n, dtype=torch.float32 if k in ("rho", "delta") else torch.int32, device="cuda")
               for k in KEYS_2D}
        algo.run_batch(np.array([0, n], np.int64), dev["x"], dev["y"], dev["layer"], dev["weight"], out=out,
                       flags=C.DEVICE_MEMORY)
        algo.synchronize()
        assert_bitexact({k: v.cpu().numpy() for k, v in out.items()}, want)
    algo.close()
