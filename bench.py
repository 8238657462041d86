"""Benchmark of the GB300 CLUE path (one JSON line on stdout from rank 0).

Default workload: batched CLUE 2D over 4096 synthetic HGCAL-like events whose
sizes are log-uniform in [5k, 200k] points (216M points, 3.5 GB of inputs,
far larger than the 129 MB L2, so no flush is needed between steps).

* ``value``: events/s of the batched path (one CUDA-graph replay per step),
  inputs and outputs resident in HBM, CUDA events on the launching stream.
* ``e2e``: the same through the C ABI with host (pinned) buffers, H2D of the
  inputs and D2H of all five outputs inside every step; ``e2e.copy_floor``
  times the same copies without the kernels right after, in the pipelined
  path's sub-batches and as whole arrays (the host link's floor on this machine).
* ``roofline``: the dominant kernel (k_layers), timed per stage with CUDA
  events on its stream in a second pass over the same workload; algorithmic
  bytes = 80 B per point (the reference's four stages each streaming their
  SoA inputs once and writing their outputs once).
* ``plain_*``: the same kernels one event per launch sequence.
* ``cpu_baseline``: the reference's own serial algorithm
  (``CLUEAlgoSerial::makeClusters``, compiled from its unmodified sources by
  ``oracle/build.py`` into ``oracle/_ref``) over all host cores on a bounded
  sample, kind "reference"; the oracle port (a C restatement, bit-identical)
  is timed beside it, and stands in (kind "port") where the reference's
  sources were not available to build.
* ``serving``: Poisson arrivals into the continuous-batching server and into
  a one-event server, at a fixed load and at a load above the latter's
  capacity; ``clue3d``: batched CLUE3D on 1,000 events of layer clusters;
  ``hgcal_1000``: batched and plain on 1,000 HGCAL-occupancy events (about
  325k points each), and the chain 2D -> bridge -> CLUE3D on them.

``--impl reference`` times that CPU implementation alone on the same
workload and prints the reference arm's line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "heterogeneous-clue_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "CLUE events/s & Gpoints/s, batched vs plain on 1 GB300 (bit-exact); p99 latency"
BYTES_PER_POINT = 80          # algorithmic bytes per point, all four stages
COMPULSORY_BYTES_PER_POINT = 36
PARAMS = (1.3, 2.0, 2.0)
# DRAM bytes per point of k_layers (both passes of one batch), from an ncu capture
# of the 256-event uneven batch (dram read + write over its 13,628,373 points);
# traffic grows with the point count, so a full launch is scaled by its points.
K_LAYERS_DRAM_BYTES_PER_POINT = 24.44
# Warp instructions per point of k_layers (both passes), same capture: the
# kernel is bound by instruction issue, so its issue rate against the SMs'
# peak (4 schedulers x 1 instruction per cycle) is the bound that applies.
K_LAYERS_WARP_INST_PER_POINT = 96.99
# Where the two figures come from (reported with them in the JSON line).
K_LAYERS_CAPTURE = {"commit": "ab43302", "summary": "profiles/k_layers_uneven256.md",
                    "workload": "256-event uneven batch, 13,628,373 points, both passes"}



def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def gen_workload(args, rank):
    from clue_gb300 import synthetic as S
    if args.workload in ("batched", "plain"):
        return S.uneven_batch(args.events, seed=7 + 1000 * rank)
    raise ValueError(args.workload)


def cpu_sample(b, n_sample):
    import numpy as np
    E = b["offsets"].size - 1
    idx = np.linspace(0, E - 1, min(n_sample, E)).astype(np.int64)
    idx = np.unique(idx)
    parts = {k: [] for k in ("x", "y", "layer", "weight")}
    sizes = []
    for e in idx:
        s, t = b["offsets"][e], b["offsets"][e + 1]
        for k in parts:
            parts[k].append(b[k][s:t])
        sizes.append(t - s)
    off = np.zeros(len(sizes) + 1, np.int64)
    np.cumsum(sizes, out=off[1:])
    return dict(offsets=off, **{k: np.concatenate(v) for k, v in parts.items()})


def cpu_kind():
    """"reference" when the unmodified reference can be built here (from its
    tree or its install under baseline/_ref), else "port"."""
    import oracle
    try:
        oracle.ref_lib()
        return "reference"
    except Exception:
        return "port"


def time_cpu(b, n_sample, threads, kind="port"):
    """CPU throughput on a strided sample of the workload: the reference's own
    CLUEAlgoSerial::makeClusters (kind "reference", one algorithm object per
    thread, timed around the makeClusters calls) or the oracle port (kind
    "port", timed around the whole batch call)."""
    import oracle
    smp = cpu_sample(b, n_sample)
    args = (smp["offsets"], smp["x"], smp["y"], smp["layer"], smp["weight"], *PARAMS)
    if kind == "reference":
        _, dt = oracle.ref_clue2d_batch(*args, n_threads=threads)
    else:
        t0 = time.perf_counter()
        oracle.clue2d_batch(*args, n_threads=threads)
        dt = time.perf_counter() - t0
    ev = smp["offsets"].size - 1
    return dict(events=ev, points=int(smp["offsets"][-1]), seconds=dt, events_per_s=ev / dt,
                gpoints_per_s=smp["offsets"][-1] / dt / 1e9)


def time_cpu_single(reps=3, kind="port"):
    """Single-thread latency of the CPU implementation on one toy-detector
    event (100k points) and one HGCAL-occupancy event (about 325k points):
    the best of ``reps`` runs, input generation excluded."""
    import numpy as np

    import oracle
    from clue_gb300 import synthetic as S
    res = {}
    for name, ev in (("toy_100k", S.toy_event(12345)), ("hgcal_event", S.hgcal_event(1000))):
        best = float("inf")
        off = np.array([0, ev["x"].size], np.int64)
        for _ in range(reps):
            if kind == "reference":
                _, dt = oracle.ref_clue2d_batch(off, ev["x"], ev["y"], ev["layer"], ev["weight"], *PARAMS)
            else:
                t0 = time.perf_counter()
                oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *PARAMS)
                dt = time.perf_counter() - t0
            best = min(best, dt)
        res[name] = {"points": int(ev["x"].size), "ms": 1000.0 * best}
    return res


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    b = gen_workload(args, 0)
    threads = os.cpu_count() or 1
    kind = cpu_kind()
    for _ in range(args.warmup):
        time_cpu(b, max(8, args.cpu_sample // 8), threads, kind)
    secs, evs, pts = 0.0, 0, 0
    for _ in range(args.steps):
        r = time_cpu(b, args.cpu_sample, threads, kind)
        secs += r["seconds"]
        evs += r["events"]
        pts += r["points"]
    v = evs / secs
    sample = (f"{evs // max(args.steps, 1)} events strided over the {args.events}-event workload "
              f"({pts // max(args.steps, 1)} points) per step")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "events/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded HGCAL-like generator)",
            "config": _config(args, b),
            "gpoints_per_s": pts / secs / 1e9,
            "cpu_baseline": {"value": v, "unit": "events/s", "cores": threads, "kind": kind, "sample": sample,
                             "implementation": ("CLUEAlgoSerial::makeClusters, unmodified reference sources"
                                                if kind == "reference" else "oracle port (C restatement)")},
            "e2e": {"value": v, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _config(args, b):
    import numpy as np
    sizes = np.diff(b["offsets"])
    return {"workload": f"batched CLUE 2D, {args.events} events, sizes log-uniform 5k-200k points",
            "events": int(sizes.size), "points": int(b["offsets"][-1]),
            "points_per_event_min_mean_max": [int(sizes.min()), float(sizes.mean()), int(sizes.max())],
            "dc": PARAMS[0], "rhoc": PARAMS[1], "outlierDeltaFactor": PARAMS[2], "layers": 100,
            "l2": "inputs (16 B/point) larger than L2; no flush"}


def serving_leg(C, b, rate, n_req, batched=True):
    """Poisson arrivals of events from the workload at ``rate`` events/s into
    the continuous-batching server (batched) or into a one-event-per-launch
    server (plain: one batch of one event in flight); latency is submit ->
    outputs written, measured by the server.  Requests are consecutive events
    of the workload; the client submits every request whose arrival time has
    passed in one bulk call (``submit_many``), so that the offered load is not
    capped by the submitting thread."""
    import numpy as np

    E = b["offsets"].size - 1
    off = b["offsets"]
    rng = np.random.default_rng(5)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    srv = C.Server(*PARAMS, budget_bytes=16 << 30, max_inflight=2 if batched else 1,
                   max_batch_events=256 if batched else 1)

    def submit(i, j):  # requests i..j-1 = events i % E .. (j - 1) % E, no wrap inside
        e0 = i % E
        s, t = off[e0], off[e0 + (j - i)]
        sub = off[e0:e0 + (j - i) + 1] - s
        return srv.submit_many(sub, b["x"][s:t], b["y"][s:t], b["layer"][s:t], b["weight"][s:t])

    # warm the slots (first launches, single and multi-event batches) outside the measurement
    warm = submit(0, 1) + submit(1, 2) + submit(2, min(18, n_req))
    srv.drain()
    for rid, _ in warm:
        srv.poll(rid, 0)
    srv.reset_stats()
    t0 = time.perf_counter()
    ids = []
    i = 0
    while i < n_req:
        now = time.perf_counter() - t0
        j = int(np.searchsorted(arrivals, now, side="right"))
        if j > i:
            j = min(j, i + (E - i % E))  # a burst never wraps around the workload
            ids += submit(i, j)
            i = j
            continue
        wait = arrivals[i] - now
        if wait > 0.002:
            time.sleep(wait - 0.001)
    srv.drain()
    elapsed = time.perf_counter() - t0
    st = srv.stats()
    for rid, _ in ids:
        srv.poll(rid, 0)
    srv.close()
    pts = int(sum(int(off[(k % E) + 1] - off[k % E]) for k in range(n_req)))
    return {"offered_events_per_s": rate, "requests": n_req, "achieved_events_per_s": n_req / elapsed,
            "achieved_gpoints_per_s": pts / elapsed / 1e9, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
            "mean_batch_events": st["mean_batch_events"], "max_inflight_seen": st["max_inflight_seen"],
            "budget_bytes": 16 << 30, "max_inflight": 2 if batched else 1}


PIPE_POINTS = 8 << 20  # sub-batch size of the library's pipelined host-memory path


def copy_floor(torch, off, hin, hout, dev_in, reps=3):
    """The e2e step's copies alone, with no kernels: the same arrays in the
    same event-aligned sub-batches of about PIPE_POINTS points as the
    pipelined path (inputs on one stream, outputs on another, overlapped), and
    the same bytes as one copy per array.  The pipelined e2e step cannot beat
    the first; the host link's shared bandwidth sets both."""
    E = len(off) - 1
    cut = [0]
    for e in range(E):
        if off[e + 1] - off[cut[-1]] >= PIPE_POINTS and e + 1 < E:
            cut.append(e + 1)
    cut.append(E)
    dev_out = {k: torch.empty(v.numel(), dtype=v.dtype, device="cuda") for k, v in hout.items()}
    si, so = torch.cuda.Stream(), torch.cuda.Stream()

    def chunked():
        with torch.cuda.stream(si):
            for i in range(len(cut) - 1):
                p0, p1 = int(off[cut[i]]), int(off[cut[i + 1]])
                for k, v in hin.items():
                    dev_in[k][p0:p1].copy_(v[p0:p1], non_blocking=True)
        with torch.cuda.stream(so):
            for i in range(len(cut) - 1):
                p0, p1 = int(off[cut[i]]), int(off[cut[i + 1]])
                for k, v in hout.items():
                    v[p0:p1].copy_(dev_out[k][p0:p1], non_blocking=True)

    def whole():
        with torch.cuda.stream(si):
            for k, v in hin.items():
                dev_in[k].copy_(v, non_blocking=True)
        with torch.cuda.stream(so):
            for k, v in hout.items():
                v.copy_(dev_out[k], non_blocking=True)

    res = {}
    for name, f in (("sub_batches", chunked), ("whole_arrays", whole)):
        ts = []
        for r in range(reps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            f()
            torch.cuda.synchronize()
            if r:
                ts.append(1000 * (time.perf_counter() - t0))
        res[name + "_ms"] = statistics.median(ts)
    nbytes = sum(v.numel() * v.element_size() for v in list(hin.values()) + list(hout.values()))
    res["bytes"] = nbytes
    res["sub_batches"] = len(cut) - 1
    res["sub_batches_gb_per_s"] = nbytes / res["sub_batches_ms"] / 1e6
    res["whole_arrays_gb_per_s"] = nbytes / res["whole_arrays_ms"] / 1e6
    del dev_out
    return res


def config2_leg(C, torch, stream, args):
    """HGCAL-occupancy events (100 layers x 50 blobs of 30-80 points + 500
    noise points per layer, about 325k points each, seeds 1000 + e): the
    batched form (device resident, graph replay) and the plain form (one
    event per launch sequence) of the same kernels on the same events."""
    from clue_gb300 import synthetic as S
    b = S.hgcal_batch(args.config2_events, seed=1000)
    off = b["offsets"]
    E, N = off.size - 1, int(off[-1])
    dev = {k: torch.from_numpy(b[k]).cuda() for k in ("x", "y", "layer", "weight")}
    out = {k: torch.empty(N, dtype=torch.float32 if k in ("rho", "delta") else torch.int32, device="cuda")
           for k in ("rho", "delta", "nearestHigher", "isSeed", "clusterIndex")}
    algo = C.Clusterizer(*PARAMS, budget_bytes=96 << 30, stream=stream.cuda_stream)
    if not args.no_autotune:
        # denser layers than the main workload: the decomposition is tuned for them
        import tempfile
        algo.autotune(off, dev["x"], dev["y"], dev["layer"], dev["weight"], out,
                      cache_path=os.path.join(tempfile.gettempdir(), "clue_gb300_autotune.jsonl"))

    def run(h, flags):
        h.run_batch(off, dev["x"], dev["y"], dev["layer"], dev["weight"], out=out, flags=C.DEVICE_MEMORY | flags)

    def timed(h, flags, warm, steps):
        """Per-step times (ms, CUDA events on the stream) of ``steps`` steps after ``warm``."""
        for _ in range(warm):
            run(h, flags)
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            run(h, flags)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        h.synchronize()
        return ts

    steps = max(5, args.steps)
    tb = timed(algo, 0, 3, steps)
    # the plain form on a handle of its own with the same tuning: on the handle
    # the autotuner ran on, one-event runs measured up to 1.5x slower
    plain_h = C.Clusterizer(*PARAMS, budget_bytes=96 << 30, stream=stream.cuda_stream)
    t = algo.get_tuning()
    plain_h.set_tuning(threads=t["threads"], layer_capacity=t["layer_capacity"], big_threads=t["big_threads"],
                       big_capacity=t["big_capacity"])
    tp = timed(plain_h, C.PLAIN, 2, steps)
    plain_h.close()
    ms_b, ms_p = statistics.median(tb), statistics.median(tp)
    tuning = algo.get_tuning()
    chain = None if args.no_chain else chain_leg(C, torch, stream, algo, off, dev, out, steps)
    algo.close()
    del dev, out
    torch.cuda.empty_cache()
    res = {"events": E, "points": N, "steps": steps, "batched_events_per_s": E / (ms_b / 1000.0),
           "batched_gpoints_per_s": N / (ms_b / 1000.0) / 1e9, "plain_events_per_s": E / (ms_p / 1000.0),
           "batched_over_plain": ms_p / ms_b,
           "batched_over_plain_min_median_max": [min(tp) / max(tb), ms_p / ms_b, max(tp) / min(tb)],
           "batched_ms_min_median_max": [min(tb), ms_b, max(tb)],
           "plain_ms_min_median_max": [min(tp), ms_p, max(tp)], "tuning": tuning}
    return res, chain


def chain_leg(C, torch, stream, algo, off, dev, out, steps):
    """CLUE3D on the layer clusters of the 1,000 HGCAL-occupancy events: CLUE
    2D (device resident), the 2D -> 3D bridge on the device (layer clusters
    from the 2D clusters), then batched CLUE3D (100 layers, +-2 sibling
    layers, criticalDensity 0.5) on the bridge's output.  Events/s of the
    chain and each stage's share; stage times are CUDA events on the stream,
    which also cover the bridge's read of the per-event cluster counts."""
    prm3 = dict(n_layers=100, density_sibling_layers=2, nh_sibling_layers=2, critical_density=0.5)
    out3 = None
    E = off.size - 1

    def step():
        nonlocal out3
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        t0 = time.perf_counter()
        ev[0].record(stream)
        algo.run_batch(off, dev["x"], dev["y"], dev["layer"], dev["weight"], out=out, flags=C.DEVICE_MEMORY)
        ev[1].record(stream)
        coff, lc = algo.layer_clusters(off, dev["x"], dev["y"], dev["layer"], dev["weight"], out)
        ev[2].record(stream)
        n3 = int(coff[-1])
        if out3 is None or out3["rho"].numel() != n3:
            out3 = {k: torch.empty(n3, dtype=torch.float32 if k in ("rho", "delta_transverse") else torch.int32,
                                   device="cuda")
                    for k in ("rho", "delta_transverse", "delta_layers", "nh_layer", "nh_index", "isSeed",
                              "tracksterIndex")}
        algo.run_clue3d(coff, lc, params=prm3, flags=C.DEVICE_MEMORY, out=out3)
        ev[3].record(stream)
        torch.cuda.synchronize()
        algo.synchronize()
        wall = (time.perf_counter() - t0) * 1000.0
        return [ev[i].elapsed_time(ev[i + 1]) for i in range(3)], wall, n3

    for _ in range(2):
        step()
    rows = [step() for _ in range(steps)]
    tot = [sum(r[0]) for r in rows]
    med = statistics.median(tot)
    stage = {name: statistics.median([r[0][i] for r in rows]) for i, name in enumerate(("clue2d", "bridge", "clue3d"))}
    wall = statistics.median([r[1] for r in rows])
    return {"events": E, "layer_clusters": rows[-1][2], "steps": steps, "events_per_s": E / (med / 1000.0),
            "ms_per_step": med, "wall_ms_per_step": wall, "stage_ms": stage,
            "stage_share": {k: v / med for k, v in stage.items()},
            "clue3d_params": prm3, "bridge": "energy = sum of weights, x/y weighted means, layer_z 320-520 cm, "
                                             "radius 2 cm, isSilicon 1"}


def clue3d_leg(C, torch, stream, args):
    """Batched CLUE3D on synthetic layer clusters: 1000 events of 2k-20k
    clusters, 100 layers, +-2 sibling layers, criticalDensity 0.5."""
    import numpy as np

    from clue_gb300 import synthetic as S
    b3 = S.clue3d_batch(args.clue3d_events, seed0=1000, n_layers=100)
    off = b3["offsets"]
    n = int(off[-1])
    prm = dict(n_layers=100, density_sibling_layers=2, nh_sibling_layers=2, critical_density=0.5)
    fields = ("z", "eta", "phi", "r_over_absz", "radius", "layer", "energy", "isSilicon")
    dev = {k: torch.from_numpy(np.ascontiguousarray(b3[k])).cuda() for k in fields}
    out = {k: torch.empty(n, dtype=torch.float32 if k in ("rho", "delta_transverse") else torch.int32,
                          device="cuda")
           for k in ("rho", "delta_transverse", "delta_layers", "nh_layer", "nh_index", "isSeed", "tracksterIndex")}
    algo = C.Clusterizer(*PARAMS, budget_bytes=32 << 30, stream=stream.cuda_stream)
    for _ in range(2):
        algo.run_clue3d(off, dev, params=prm, flags=C.DEVICE_MEMORY, out=out)
    algo.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(3, args.steps)
    e0.record(stream)
    for _ in range(steps):
        algo.run_clue3d(off, dev, params=prm, flags=C.DEVICE_MEMORY, out=out)
    e1.record(stream)
    torch.cuda.synchronize()
    algo.synchronize()
    ms = e0.elapsed_time(e1) / steps
    algo.close()
    peak, _ = _peak_hbm()
    achieved = 92 * n / (ms / 1000.0) / 1e9
    return {"events": int(off.size - 1), "layer_clusters": n, "ms_per_step": ms,
            "events_per_s": (off.size - 1) / (ms / 1000.0), "mclusters_per_s": n / (ms / 1000.0) / 1e6,
            "params": prm, "roofline": {"algorithmic_bytes_per_cluster": 92, "achieved_gbs": achieved,
                                        "peak_gbs": peak, "frac": achieved / peak}}


def run_gb300(args):
    import numpy as np
    import torch

    import clue_gb300 as C

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    b = gen_workload(args, rank)
    E = b["offsets"].size - 1
    N = int(b["offsets"][-1])
    stream = torch.cuda.Stream()
    algo = C.Clusterizer(*PARAMS, budget_bytes=96 << 30, device=local, stream=stream.cuda_stream)
    if args.tuning:
        algo.set_tuning(**json.loads(args.tuning))
    dev = {k: torch.from_numpy(b[k]).cuda() for k in ("x", "y", "layer", "weight")}
    out = dict(rho=torch.empty(N, dtype=torch.float32, device="cuda"),
               delta=torch.empty(N, dtype=torch.float32, device="cuda"),
               nearestHigher=torch.empty(N, dtype=torch.int32, device="cuda"),
               isSeed=torch.empty(N, dtype=torch.int32, device="cuda"),
               clusterIndex=torch.empty(N, dtype=torch.int32, device="cuda"))
    off = b["offsets"]
    if not args.tuning and not args.no_autotune:
        # the project's autotuner picks the work decomposition on this workload
        # (all candidates are checked to give identical outputs)
        import tempfile
        algo.autotune(off, dev["x"], dev["y"], dev["layer"], dev["weight"], out,
                      cache_path=os.path.join(tempfile.gettempdir(), "clue_gb300_autotune.jsonl"))

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    def max_over_ranks(v):
        return C.dist_max(v, device="cuda")

    def run(flags):
        algo.run_batch(off, dev["x"], dev["y"], dev["layer"], dev["weight"], out=out, flags=C.DEVICE_MEMORY | flags)

    # ---- batched, device resident (headline value)
    for _ in range(args.warmup):
        run(0)
    # kernels per step as the library counted them (the graph's kernels)
    launches_per_step = algo.last_run_stats()["kernel_launches"]
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # clocks are sampled over the timed steps and the per-stage pass that follows
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            run(0)
        ev1.record(stream)
        torch.cuda.synchronize()
        algo.synchronize()
        barrier()

        # ---- per-stage times of the same workload (roofline of the dominant kernel)
        stage_sum = {s: 0.0 for s in C.STAGES}
        prof_steps = max(1, min(args.steps, 5))
        for _ in range(prof_steps):
            st = algo.profile_batch(off, dev["x"], dev["y"], dev["layer"], dev["weight"], out)
            for k, v in st.items():
                stage_sum[k] += v
    ms = max_over_ranks(ev0.elapsed_time(ev1))
    ms_step = ms / args.steps
    value = ws * E * args.steps / (ms / 1000.0)
    gpts = ws * N * args.steps / (ms / 1000.0) / 1e9
    stage_ms = {k: v / prof_steps for k, v in stage_sum.items()}
    peak, peak_kind = _peak_hbm()
    layers_ms = stage_ms["layers"]
    clocks = clk.summary()
    achieved = BYTES_PER_POINT * N / (layers_ms / 1000.0) / 1e9
    pipe_achieved = BYTES_PER_POINT * N / (ms_step / 1000.0) / 1e9
    traffic = K_LAYERS_DRAM_BYTES_PER_POINT * N
    roofline = {"bound": "hbm", "kernel": "k_layers", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_point": BYTES_PER_POINT,
                "pipeline_achieved": pipe_achieved, "pipeline_frac": pipe_achieved / peak,
                "compulsory_frac": COMPULSORY_BYTES_PER_POINT * N / (ms_step / 1000.0) / 1e9 / peak}
    props = torch.cuda.get_device_properties(local)
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    issue_peak = props.multi_processor_count * 4 * mhz * 1e6
    issue_achieved = K_LAYERS_WARP_INST_PER_POINT * N / (layers_ms / 1000.0)
    roofline["traffic_source"] = K_LAYERS_CAPTURE
    roofline["issue"] = {"warp_instructions_per_point": K_LAYERS_WARP_INST_PER_POINT,
                         "achieved_warp_inst_per_s": issue_achieved, "peak_warp_inst_per_s": issue_peak,
                         "frac": issue_achieved / issue_peak, "sm_mhz": mhz}

    # ---- plain: the same kernels, one event per launch sequence
    plain = plain_spread = None
    if not args.no_plain:
        run(C.PLAIN)
        torch.cuda.synchronize()
        pts_ms = []
        for _ in range(max(3, args.steps // 3)):
            p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            p0.record(stream)
            run(C.PLAIN)
            p1.record(stream)
            torch.cuda.synchronize()
            pts_ms.append(max_over_ranks(p0.elapsed_time(p1)))
        pms = statistics.median(pts_ms)
        plain = ws * E / (pms / 1000.0)
        plain_spread = {"plain_ms_min_median_max": [min(pts_ms), pms, max(pts_ms)], "steps": len(pts_ms),
                        "batched_over_plain_min_median_max": [min(pts_ms) / ms_step, pms / ms_step,
                                                              max(pts_ms) / ms_step]}

    # ---- serving, before the e2e leg: run after it (which leaves 7.8 GB of pinned
    # buffers in torch's host cache), the servers' p99 at 2,000 events/s measured
    # 4.2 ms instead of 1.6 ms
    serving = None
    if rank == 0 and not args.no_serving:
        serving = {"batched": serving_leg(C, b, args.serving_rate, args.serving_requests, batched=True),
                   "plain": serving_leg(C, b, args.serving_rate, max(200, args.serving_requests // 4),
                                        batched=False)}
        if args.serving_high_rate > 0:
            # above the one-event server's capacity: batches form, the plain queue grows
            serving["high_load"] = {
                "batched": serving_leg(C, b, args.serving_high_rate, args.serving_requests, batched=True),
                "plain": serving_leg(C, b, args.serving_high_rate, max(200, args.serving_requests // 4),
                                     batched=False)}

    # ---- end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        del out
        hin = {k: torch.from_numpy(b[k]).pin_memory() for k in ("x", "y", "layer", "weight")}
        hout = dict(rho=torch.empty(N, dtype=torch.float32).pin_memory(),
                    delta=torch.empty(N, dtype=torch.float32).pin_memory(),
                    nearestHigher=torch.empty(N, dtype=torch.int32).pin_memory(),
                    isSeed=torch.empty(N, dtype=torch.int32).pin_memory(),
                    clusterIndex=torch.empty(N, dtype=torch.int32).pin_memory())
        for _ in range(max(1, args.warmup)):
            algo.run_batch(off, hin["x"], hin["y"], hin["layer"], hin["weight"], out=hout)
        barrier()
        step_ms = []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            t1 = time.perf_counter()
            algo.run_batch(off, hin["x"], hin["y"], hin["layer"], hin["weight"], out=hout)
            step_ms.append(1000 * (time.perf_counter() - t1))
        dt = max_over_ranks(time.perf_counter() - t0)
        st = algo.last_run_stats()  # the copies as the library made them
        h2d_bytes, d2h_bytes = st["h2d_bytes"], st["d2h_bytes"]
        e2e = {"value": ws * E * args.steps / dt, "unit": "events/s",
               "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h_bytes,
               "gpoints_per_s": ws * N * args.steps / dt / 1e9, "ms_per_step": 1000 * dt / args.steps,
               "step_ms_min_median_max": [min(step_ms), statistics.median(step_ms), max(step_ms)],
               "step_ms": [round(t, 3) for t in step_ms]}
        # the same copies without the kernels, right after the timed steps
        e2e["copy_floor"] = copy_floor(torch, off, hin, hout, dev)
        del hin, hout

    # the legs below use handles of their own: release the main one's buffers
    t_main = algo.get_tuning()
    algo.close()
    del dev
    if args.no_e2e:
        del out
    torch.cuda.empty_cache()

    clue3d = None
    if rank == 0 and not args.no_clue3d:
        clue3d = clue3d_leg(C, torch, stream, args)
    # ---- one event alone: the reference producer's call (toy-detector event, 100k points)
    single = None
    if rank == 0:
        from clue_gb300 import synthetic as S
        ev = S.toy_event(12345)
        n1 = ev["x"].size
        one = C.Clusterizer(*PARAMS, budget_bytes=4 << 30, stream=stream.cuda_stream)
        for _ in range(3):
            one.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
        t0 = time.perf_counter()
        for _ in range(20):
            one.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
        host_ms = (time.perf_counter() - t0) / 20 * 1000.0
        d1 = {k: torch.from_numpy(ev[k]).cuda() for k in ("x", "y", "layer", "weight")}
        o1 = {k: torch.empty(n1, dtype=torch.float32 if k in ("rho", "delta") else torch.int32, device="cuda")
              for k in ("rho", "delta", "nearestHigher", "isSeed", "clusterIndex")}
        off1 = np.array([0, n1], np.int64)
        for _ in range(3):
            one.run_batch(off1, d1["x"], d1["y"], d1["layer"], d1["weight"], out=o1, flags=C.DEVICE_MEMORY)
        one.synchronize()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        for _ in range(20):
            one.run_batch(off1, d1["x"], d1["y"], d1["layer"], d1["weight"], out=o1, flags=C.DEVICE_MEMORY)
        s1.record(stream)
        torch.cuda.synchronize()
        one.synchronize()
        one.close()
        single = {"event": "toy-detector, 100,000 points", "host_memory_ms": host_ms,
                  "device_memory_ms": s0.elapsed_time(s1) / 20}

    config2 = chain = None
    if rank == 0 and not args.no_config2:
        config2, chain = config2_leg(C, torch, stream, args)

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        kind = cpu_kind()
        r = time_cpu(b, args.cpu_sample, threads, kind)
        cpu = {"value": r["events_per_s"], "unit": "events/s", "cores": threads, "kind": kind,
               "sample": f"{r['events']} events strided over the workload ({r['points']} points), "
                         f"{r['seconds']:.1f} s on {threads} threads",
               "gpoints_per_s": r["gpoints_per_s"], "single_thread_latency": time_cpu_single(kind=kind)}
        if kind == "reference":
            # the oracle port on the same sample, for comparison
            rp = time_cpu(b, args.cpu_sample, threads, "port")
            cpu["port"] = {"value": rp["events_per_s"], "unit": "events/s", "cores": threads,
                           "seconds": rp["seconds"]}

    if rank == 0:
        # the ratios and the end-to-end figure first: a truncated line still shows them
        line = {"metric": METRIC, "value": value, "unit": "events/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded HGCAL-like generator)",
                "gpoints_per_s": gpts,
                "plain_events_per_s": plain, "batched_over_plain": (value / plain) if plain else None,
                "plain_spread": plain_spread,
                "hgcal_1000_batched_over_plain": (config2["batched_over_plain_min_median_max"]
                                                  if config2 else None),
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
                "gpu_launches": launches_per_step * args.steps,
                "config": _config(args, b), "stage_ms": stage_ms,
                "clue3d": clue3d, "clue3d_from_config2": chain, "hgcal_1000": config2,
                "serving": serving, "single_event": single, "tuning": t_main}
        print(json.dumps(line), flush=True)
    algo.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched", choices=["batched"])
    ap.add_argument("--events", type=int, default=4096)
    ap.add_argument("--cpu-sample", type=int, default=512)
    ap.add_argument("--tuning", default="")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serving-rate", type=float, default=2000.0)
    ap.add_argument("--serving-high-rate", type=float, default=20000.0,
                    help="second offered load (events/s) above the plain server's capacity; 0 = skip")
    ap.add_argument("--serving-requests", type=int, default=3000)
    ap.add_argument("--no-clue3d", action="store_true")
    ap.add_argument("--no-config2", action="store_true",
                    help="skip the batched-vs-plain measurement on HGCAL-occupancy events")
    ap.add_argument("--config2-events", type=int, default=1000)
    ap.add_argument("--no-chain", action="store_true",
                    help="skip CLUE 2D -> bridge -> CLUE3D on the HGCAL-occupancy events")
    ap.add_argument("--clue3d-events", type=int, default=1000)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
