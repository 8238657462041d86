"""Python front end of libclue_gb300.so (ctypes over the C ABI in include/clue.h).

The product is the C ABI and the CUDA kernels behind it; this module only
binds them for Python callers, tests and the benchmark.  There is no CPU
fallback: every call goes to the GPU library, and loading fails loudly when
the library was not built.

``Clusterizer.make_clusters`` mirrors the reference producer's call
``CLUEAlgoSerial::makeClusters(PointsCloud const&, PointsCloudSerial&, dc,
rhoc, outlierDeltaFactor)`` (src/serial/plugin-CLUEClusterizer/CLUEAlgoSerial.h:13):
PointsCloud arrays in, the PointsCloudSerial output arrays out.
"""
import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "lib", "libclue_gb300.so")
HEADER = os.path.join(ROOT, "include", "clue.h")

STAGES = ("count", "layer_scan", "scatter", "layers", "seed_chunk_scan", "seed_rank", "label")

CLUE_OK, CLUE_EINVAL, CLUE_ENOMEM, CLUE_ECUDA, CLUE_ETIMEOUT, CLUE_EBUSY = range(6)
HOST_MEMORY, DEVICE_MEMORY, PLAIN, NO_GRAPH, NO_PIPELINE = 0, 1, 2, 4, 8

_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p


class ClueError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("dc", ctypes.c_float), ("rhoc", ctypes.c_float), ("outlierDeltaFactor", ctypes.c_float)]


class Outputs(ctypes.Structure):
    _fields_ = [("rho", _vp), ("delta", _vp), ("nearestHigher", _vp), ("isSeed", _vp), ("clusterIndex", _vp)]


class Tuning(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int32), ("layer_capacity", ctypes.c_int32),
                ("work_tile_cm", ctypes.c_float), ("ctas_per_sm", ctypes.c_int32),
                ("big_threads", ctypes.c_int32), ("big_capacity", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Params3D(ctypes.Structure):
    _fields_ = [
        ("n_layers", ctypes.c_int32), ("density_sibling_layers", ctypes.c_int32),
        ("density_xy_distance_sqr", ctypes.c_float), ("kernel_density_factor", ctypes.c_float),
        ("density_on_same_layer", ctypes.c_int32), ("nh_sibling_layers", ctypes.c_int32),
        ("nh_on_same_layer", ctypes.c_int32), ("critical_xy_distance", ctypes.c_float),
        ("critical_z_distance_lyr", ctypes.c_float), ("critical_density", ctypes.c_float),
        ("critical_self_density", ctypes.c_float), ("outlier_multiplier", ctypes.c_float)]


class Inputs3D(ctypes.Structure):
    _fields_ = [(k, _vp) for k in ("z", "eta", "phi", "r_over_absz", "radius", "layer", "energy", "isSilicon")]


class Outputs3D(ctypes.Structure):
    _fields_ = [(k, _vp) for k in ("rho", "delta_transverse", "delta_layers", "nh_layer", "nh_index", "isSeed",
                                   "tracksterIndex")]


class BridgeParams(ctypes.Structure):
    _fields_ = [("n_layers", ctypes.c_int32), ("layer_z", _vp), ("radius", ctypes.c_float),
                ("isSilicon", ctypes.c_int32)]


LAYER_CLUSTER_FIELDS = ("x", "y", "z", "eta", "phi", "r_over_absz", "radius", "layer", "energy", "isSilicon")


class LayerClusters(ctypes.Structure):
    _fields_ = [(k, _vp) for k in LAYER_CLUSTER_FIELDS]


class ServerConfig(ctypes.Structure):
    _fields_ = [("device_budget_bytes", ctypes.c_size_t), ("max_inflight", ctypes.c_int32),
                ("max_batch_events", ctypes.c_int32), ("device", ctypes.c_int32)]


class RunStats(ctypes.Structure):
    _fields_ = [("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64), ("kernel_launches", ctypes.c_int64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_int64), ("batches", ctypes.c_int64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("mean_batch_events", ctypes.c_double),
                ("max_inflight_seen", ctypes.c_double), ("slot_capacity_points", ctypes.c_int64),
                ("memory_waits", ctypes.c_int64)]


def header_symbols():
    """Function names the C ABI header declares."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|size_t|void|const char\*)\s+\**\s*(clue\w*)\s*\(", txt, re.M)))


_lib = None


def lib():
    """Load libclue_gb300.so (raises when it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} missing: run __graft_entry__.build() (no CPU fallback exists)")
    l = ctypes.CDLL(LIB_PATH)
    H = _vp
    sig = {
        "clue_last_error": ([], ctypes.c_char_p),
        "clue_create": ([ctypes.POINTER(Params), ctypes.c_size_t, ctypes.c_int, _vp, ctypes.POINTER(H)], ctypes.c_int),
        "clue_destroy": ([H], ctypes.c_int),
        "clue_set_params": ([H, ctypes.POINTER(Params)], ctypes.c_int),
        "clue_set_stream": ([H, _vp], ctypes.c_int),
        "clue_run_event": ([H, ctypes.c_int32, _vp, _vp, _vp, _vp, ctypes.POINTER(Outputs), ctypes.c_int],
                           ctypes.c_int),
        "clue_run_batch": ([H, ctypes.c_int32, _i64p, _vp, _vp, _vp, _vp, ctypes.POINTER(Outputs), ctypes.c_int],
                           ctypes.c_int),
        "clue_synchronize": ([H], ctypes.c_int),
        "clue_last_run_stats": ([H, ctypes.POINTER(RunStats)], ctypes.c_int),
        "clue_required_bytes": ([ctypes.c_int32, ctypes.c_int64, ctypes.c_int], ctypes.c_size_t),
        "clue_get_tuning": ([H, ctypes.POINTER(Tuning)], ctypes.c_int),
        "clue_profile_batch": ([H, ctypes.c_int32, _i64p, _vp, _vp, _vp, _vp, ctypes.POINTER(Outputs), _f32p],
                               ctypes.c_int),
        "clue_set_tuning": ([H, ctypes.POINTER(Tuning)], ctypes.c_int),
        "clue_autotune": ([H, ctypes.c_int32, _i64p, _vp, _vp, _vp, _vp, ctypes.POINTER(Outputs), ctypes.c_char_p,
                           ctypes.POINTER(Tuning)], ctypes.c_int),
        "clue_run_event_noalloc": ([ctypes.POINTER(Params), ctypes.c_int32, _vp, _vp, _vp, _vp,
                                    ctypes.POINTER(Outputs), _vp], ctypes.c_int),
        "clue3d_default_params": ([ctypes.POINTER(Params3D)], None),
        "clue3d_run_batch": ([H, ctypes.POINTER(Params3D), ctypes.c_int32, _i64p, ctypes.POINTER(Inputs3D),
                              ctypes.POINTER(Outputs3D), _i32p, ctypes.c_int], ctypes.c_int),
        "clue_bridge_count": ([H, ctypes.c_int32, _i64p, _vp, _i64p], ctypes.c_int),
        "clue_bridge_build": ([H, ctypes.POINTER(BridgeParams), ctypes.c_int32, _i64p, _vp, _vp, _vp, _vp, _vp, _vp,
                               _i64p, ctypes.POINTER(LayerClusters)], ctypes.c_int),
        "clue_server_create": ([ctypes.POINTER(Params), ctypes.POINTER(ServerConfig), ctypes.POINTER(H)],
                               ctypes.c_int),
        "clue_server_destroy": ([H], ctypes.c_int),
        "clue_server_submit": ([H, ctypes.c_int32, _vp, _vp, _vp, _vp, ctypes.POINTER(Outputs), _i64p],
                               ctypes.c_int),
        "clue_server_submit_many": ([H, ctypes.c_int32, _i64p, _vp, _vp, _vp, _vp, ctypes.POINTER(Outputs), _i64p],
                                    ctypes.c_int),
        "clue_server_poll": ([H, ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "clue_server_drain": ([H, ctypes.c_int32], ctypes.c_int),
        "clue_server_get_stats": ([H, ctypes.POINTER(ServerStats)], ctypes.c_int),
        "clue_server_reset_stats": ([H], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        if hasattr(l, name):
            f = getattr(l, name)
            f.argtypes = args
            f.restype = res
    _lib = l
    return l


def last_error():
    return lib().clue_last_error().decode(errors="replace")


def check(rc):
    if rc != CLUE_OK:
        raise ClueError(rc, last_error())
    return rc


def _ptr(a):
    """Data pointer of a numpy array or a torch tensor."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def empty_outputs(n):
    return dict(rho=np.empty(n, np.float32), delta=np.empty(n, np.float32),
                nearestHigher=np.empty(n, np.int32), isSeed=np.empty(n, np.int32),
                clusterIndex=np.empty(n, np.int32))


def outputs_struct(o):
    return Outputs(_ptr(o["rho"]), _ptr(o["delta"]), _ptr(o["nearestHigher"]), _ptr(o["isSeed"]),
                   _ptr(o["clusterIndex"]))


class Clusterizer:
    """A CLUE handle: the reference's per-stream producer state (one
    CLUEAlgoSerial per EDM stream) as one resident GPU context."""

    def __init__(self, dc, rhoc, outlierDeltaFactor, budget_bytes=0, device=0, stream=None):
        self._h = _vp()
        p = Params(dc, rhoc, outlierDeltaFactor)
        check(lib().clue_create(ctypes.byref(p), budget_bytes, device, stream, ctypes.byref(self._h)))

    def close(self):
        if self._h:
            lib().clue_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_params(self, dc, rhoc, outlierDeltaFactor):
        check(lib().clue_set_params(self._h, ctypes.byref(Params(dc, rhoc, outlierDeltaFactor))))

    def set_stream(self, stream=None):
        """Run later work on ``stream`` (a cudaStream_t as an int, e.g.
        ``torch.cuda.Stream().cuda_stream``); None: the handle's own stream."""
        check(lib().clue_set_stream(self._h, stream))

    def make_clusters(self, x, y, layer, weight, flags=HOST_MEMORY):
        """One event, host arrays in, host arrays out."""
        x, y, w = _c(x, np.float32), _c(y, np.float32), _c(weight, np.float32)
        layer = _c(layer, np.int32)
        n = x.size
        o = empty_outputs(n)
        os_ = outputs_struct(o)
        check(lib().clue_run_event(self._h, n, _ptr(x), _ptr(y), _ptr(layer), _ptr(w), ctypes.byref(os_), flags))
        return o

    def run_batch(self, offsets, x, y, layer, weight, out=None, flags=HOST_MEMORY):
        """Events in CSR order.  Host numpy arrays by default; with
        ``flags & DEVICE_MEMORY`` the arrays are CUDA tensors (or anything
        with ``data_ptr()``) and ``out`` must be given."""
        offsets = _c(offsets, np.int64)
        if not flags & DEVICE_MEMORY:
            x, y, weight = _c(x, np.float32), _c(y, np.float32), _c(weight, np.float32)
            layer = _c(layer, np.int32)
        if out is None:
            out = empty_outputs(int(offsets[-1]))
        os_ = outputs_struct(out)
        check(lib().clue_run_batch(self._h, offsets.size - 1, offsets.ctypes.data_as(_i64p), _ptr(x), _ptr(y),
                                   _ptr(layer), _ptr(weight), ctypes.byref(os_), flags))
        return out

    def profile_batch(self, offsets, x, y, layer, weight, out):
        """Device tensors in; returns the per-stage milliseconds of one run."""
        offsets = _c(offsets, np.int64)
        os_ = outputs_struct(out)
        ms = np.zeros(STAGES.__len__(), np.float32)
        check(lib().clue_profile_batch(self._h, offsets.size - 1, offsets.ctypes.data_as(_i64p), _ptr(x), _ptr(y),
                                       _ptr(layer), _ptr(weight), ctypes.byref(os_), ms.ctypes.data_as(_f32p)))
        return dict(zip(STAGES, ms.tolist()))

    def last_run_stats(self):
        """Copies and kernels of the last 2D run on this handle:
        {"h2d_bytes", "d2h_bytes", "kernel_launches"}."""
        st = RunStats()
        check(lib().clue_last_run_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in RunStats._fields_}

    def synchronize(self):
        check(lib().clue_synchronize(self._h))

    def get_tuning(self):
        t = Tuning()
        check(lib().clue_get_tuning(self._h, ctypes.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw):
        t = Tuning()
        check(lib().clue_get_tuning(self._h, ctypes.byref(t)))
        for k, v in kw.items():
            setattr(t, k, v)
        check(lib().clue_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, offsets, x, y, layer, weight, out, cache_path=None):
        """Device tensors in; returns the chosen tuning dict."""
        offsets = _c(offsets, np.int64)
        os_ = outputs_struct(out)
        t = Tuning()
        cp = cache_path.encode() if cache_path else None
        check(lib().clue_autotune(self._h, offsets.size - 1, offsets.ctypes.data_as(_i64p), _ptr(x), _ptr(y),
                                  _ptr(layer), _ptr(weight), ctypes.byref(os_), cp, ctypes.byref(t)))
        return t.as_dict()

    def run_clue3d(self, offsets, pts, params=None, flags=HOST_MEMORY, out=None):
        """CLUE3D over events in CSR order.  ``pts`` maps the
        ClusterCollection field names to arrays (host numpy, or device tensors
        with DEVICE_MEMORY).  Returns (outputs, per-event trackster counts)."""
        offsets = _c(offsets, np.int64)
        prm = default_params3d()
        for k, v in (params or {}).items():
            setattr(prm, k, v)
        if not flags & DEVICE_MEMORY:
            pts = {k: _c(pts[k], np.int32 if k in ("layer", "isSilicon") else np.float32)
                   for k in ("z", "eta", "phi", "r_over_absz", "radius", "layer", "energy", "isSilicon")}
        n = int(offsets[-1])
        if out is None:
            out = dict(rho=np.empty(n, np.float32), delta_transverse=np.empty(n, np.float32),
                       delta_layers=np.empty(n, np.int32), nh_layer=np.empty(n, np.int32),
                       nh_index=np.empty(n, np.int32), isSeed=np.empty(n, np.int32),
                       tracksterIndex=np.empty(n, np.int32))
        inp = Inputs3D(*[_ptr(pts[k]) for k, _ in Inputs3D._fields_])
        o3 = Outputs3D(*[_ptr(out[k]) for k, _ in Outputs3D._fields_])
        nt = np.zeros(max(offsets.size - 1, 1), np.int32)
        check(lib().clue3d_run_batch(self._h, ctypes.byref(prm), offsets.size - 1, offsets.ctypes.data_as(_i64p),
                                     ctypes.byref(inp), ctypes.byref(o3), nt.ctypes.data_as(_i32p), flags))
        return out, nt[:offsets.size - 1]


    def layer_clusters(self, offsets, x, y, layer, weight, out2d, layer_z=None, radius=2.0, is_silicon=1):
        """2D -> 3D bridge on the device: the layer clusters of a clustered
        2D batch (CUDA tensors in ``x, y, layer, weight`` and ``out2d``) as
        CLUE3D input.  Returns (cluster_offsets, dict of CUDA tensors); feed
        them to ``run_clue3d(cluster_offsets, clusters, flags=DEVICE_MEMORY)``."""
        import torch
        from .synthetic import layer_z as default_layer_z
        offsets = _c(offsets, np.int64)
        E = offsets.size - 1
        coff = np.zeros(E + 1, np.int64)
        check(lib().clue_bridge_count(self._h, E, offsets.ctypes.data_as(_i64p), _ptr(out2d["isSeed"]),
                                      coff.ctypes.data_as(_i64p)))
        lz = _c(default_layer_z() if layer_z is None else layer_z, np.float32)
        C = int(coff[-1])
        out = {k: torch.empty(C, dtype=torch.int32 if k in ("layer", "isSilicon") else torch.float32,
                              device=x.device) for k in LAYER_CLUSTER_FIELDS}
        prm = BridgeParams(lz.size, lz.ctypes.data, radius, is_silicon)
        lc = LayerClusters(*[_ptr(out[k]) if C else None for k in LAYER_CLUSTER_FIELDS])
        check(lib().clue_bridge_build(self._h, ctypes.byref(prm), E, offsets.ctypes.data_as(_i64p), _ptr(x), _ptr(y),
                                      _ptr(layer), _ptr(weight), _ptr(out2d["isSeed"]), _ptr(out2d["clusterIndex"]),
                                      coff.ctypes.data_as(_i64p), ctypes.byref(lc)))
        return coff, out


def default_params3d():
    p = Params3D()
    lib().clue3d_default_params(ctypes.byref(p))
    return p


class Server:
    """Continuous-batching server over the batched CLUE kernels."""

    def __init__(self, dc, rhoc, outlierDeltaFactor, budget_bytes=16 << 30, max_inflight=2, max_batch_events=256,
                 device=0):
        self._s = _vp()
        cfg = ServerConfig(budget_bytes, max_inflight, max_batch_events, device)
        check(lib().clue_server_create(ctypes.byref(Params(dc, rhoc, outlierDeltaFactor)), ctypes.byref(cfg),
                                       ctypes.byref(self._s)))
        self._keep = {}

    def close(self):
        if self._s:
            lib().clue_server_destroy(self._s)
            self._s = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, x, y, layer, weight, out=None):
        """Queue one event (host arrays; inputs are copied at submit).
        Returns (request id, output dict that is filled on completion)."""
        x, y, w = _c(x, np.float32), _c(y, np.float32), _c(weight, np.float32)
        layer = _c(layer, np.int32)
        n = x.size
        if out is None:
            out = empty_outputs(n)
        rid = ctypes.c_int64(0)
        os_ = outputs_struct(out)
        check(lib().clue_server_submit(self._s, n, _ptr(x), _ptr(y), _ptr(layer), _ptr(w), ctypes.byref(os_),
                                       ctypes.byref(rid)))
        self._keep[rid.value] = out
        return rid.value, out

    def submit_many(self, offsets, x, y, layer, weight):
        """Queue several events (CSR ``offsets`` over host arrays) at once so
        that they can share a batch.  Returns a list of (request id, outputs)."""
        offsets = _c(offsets, np.int64)
        x, y, w = _c(x, np.float32), _c(y, np.float32), _c(weight, np.float32)
        layer = _c(layer, np.int32)
        E = offsets.size - 1
        outs = [empty_outputs(int(offsets[e + 1] - offsets[e])) for e in range(E)]
        arr = (Outputs * max(E, 1))(*[outputs_struct(o) for o in outs])
        ids = np.zeros(max(E, 1), np.int64)
        check(lib().clue_server_submit_many(self._s, E, offsets.ctypes.data_as(_i64p), _ptr(x), _ptr(y), _ptr(layer),
                                            _ptr(w), arr, ids.ctypes.data_as(_i64p)))
        for e in range(E):
            self._keep[int(ids[e])] = outs[e]
        return [(int(ids[e]), outs[e]) for e in range(E)]

    def poll(self, rid, timeout_ms=-1):
        """(status, latency_ms): status CLUE_OK when done, CLUE_EBUSY/ETIMEOUT otherwise."""
        lat = ctypes.c_double(0.0)
        rc = lib().clue_server_poll(self._s, rid, timeout_ms, ctypes.byref(lat))
        if rc not in (CLUE_OK, CLUE_EBUSY, CLUE_ETIMEOUT):
            raise ClueError(rc, last_error())
        if rc == CLUE_OK:
            self._keep.pop(rid, None)
        return rc, lat.value

    def drain(self, timeout_ms=-1):
        check(lib().clue_server_drain(self._s, timeout_ms))

    def stats(self):
        st = ServerStats()
        check(lib().clue_server_get_stats(self._s, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def reset_stats(self):
        check(lib().clue_server_reset_stats(self._s))


# ----------------------------------------------------------------------------
# Multi-process helpers (events are independent: ranks shard them, no collective
# touches the data path)
# ----------------------------------------------------------------------------

def shard_events(offsets, rank, world):
    """Contiguous event range [e0, e1) of ``rank`` among ``world`` ranks,
    balanced by point count; the ranges cover every event exactly once."""
    offsets = np.asarray(offsets, np.int64)
    E = offsets.size - 1
    N = int(offsets[-1])
    if world <= 1:
        return 0, E

    def bound(r):
        if r <= 0:
            return 0
        if r >= world:
            return E
        return int(min(E, np.searchsorted(offsets[:-1], (N * r) // world, side="left")))

    return bound(rank), bound(rank + 1)


def shard_batch(batch, rank, world):
    """The sub-batch (rebased offsets and array views) of ``rank``'s shard."""
    e0, e1 = shard_events(batch["offsets"], rank, world)
    off = batch["offsets"]
    s, t = int(off[e0]), int(off[e1])
    out = {k: batch[k][s:t] for k in ("x", "y", "layer", "weight")}
    out["offsets"] = (off[e0:e1 + 1] - off[e0]).astype(np.int64)
    out["event_range"] = (e0, e1)
    return out


def dist_max(value, device=None):
    """Max of a float over the ranks of the default process group (gloo or
    nccl); the value itself when no group is initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
