"""ctypes front end of the oracle (test infrastructure, not product code).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
use this package: to check the CUDA path's results (and bench.py to time
the CPU baseline).
``clue2d``/``clue3d`` run the CPU restatement (oracle/clue_oracle.c);
``ref_clue2d``/``ref_clue2d_batch``/``ref_clue3d`` run the unmodified
reference serial code when oracle/_ref was built (from the reference tree or
its install under baseline/_ref).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)

_lib = None
_ref = None


class Clue3DParams(ctypes.Structure):
    """Every default argument of the reference CLUE3D kernels
    (src/serial/plugin-CLUETracksterizer/CLUE3DAlgoKernels.h:26-32,286-290,509-515)
    plus the number of layers (ticl::TileConstants::nLayers = 94)."""
    _fields_ = [
        ("n_layers", ctypes.c_int32),
        ("density_sibling_layers", ctypes.c_int32),
        ("density_xy_distance_sqr", ctypes.c_float),
        ("kernel_density_factor", ctypes.c_float),
        ("density_on_same_layer", ctypes.c_int32),
        ("nh_sibling_layers", ctypes.c_int32),
        ("nh_on_same_layer", ctypes.c_int32),
        ("critical_xy_distance", ctypes.c_float),
        ("critical_z_distance_lyr", ctypes.c_float),
        ("critical_density", ctypes.c_float),
        ("critical_self_density", ctypes.c_float),
        ("outlier_multiplier", ctypes.c_float),
    ]


REFERENCE_3D_DEFAULTS = dict(
    n_layers=94, density_sibling_layers=3, density_xy_distance_sqr=3.24, kernel_density_factor=0.2,
    density_on_same_layer=0, nh_sibling_layers=3, nh_on_same_layer=0, critical_xy_distance=1.8,
    critical_z_distance_lyr=5.0, critical_density=0.6, critical_self_density=0.15, outlier_multiplier=2.0)


def _p(a, t):
    return a.ctypes.data_as(t)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_build.ORACLE_SO):
            _build.build()
        l = ctypes.CDLL(_build.ORACLE_SO)
        l.oracle_clue2d.argtypes = [ctypes.c_int32, _f32p, _f32p, _i32p, _f32p, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, _f32p, _f32p, _i32p, _i32p, _i32p]
        l.oracle_clue2d.restype = ctypes.c_int
        l.oracle_clue2d_batch.argtypes = [ctypes.c_int32, _i64p, _f32p, _f32p, _i32p, _f32p, ctypes.c_float,
                                          ctypes.c_float, ctypes.c_float, _f32p, _f32p, _i32p, _i32p, _i32p,
                                          ctypes.c_int32]
        l.oracle_clue2d_batch.restype = ctypes.c_int
        l.oracle_clue3d.argtypes = [ctypes.c_int32] + [_f32p] * 5 + [_i32p, _f32p, _i32p,
                                                                     ctypes.POINTER(Clue3DParams),
                                                                     _f32p, _f32p, _i32p, _i32p, _i32p, _i32p,
                                                                     _i32p]
        l.oracle_clue3d.restype = ctypes.c_int
        l.oracle_clue3d_batch.argtypes = ([ctypes.c_int32, _i64p] + [_f32p] * 5 + [_i32p, _f32p, _i32p,
                                                                                   ctypes.POINTER(Clue3DParams)]
                                          + [_f32p, _f32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p,
                                             ctypes.c_int32])
        l.oracle_clue3d_batch.restype = ctypes.c_int
        _lib = l
    return _lib


def ref_available():
    return os.path.exists(_build.REF_SO) or _build.ref_cmd() is not None


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(_build.REF_SO):
            _build.build()
        if not os.path.exists(_build.REF_SO):
            raise RuntimeError("reference harness not built (reference tree absent)")
        l = ctypes.CDLL(_build.REF_SO)
        l.ref_clue2d.argtypes = [ctypes.c_int32, _f32p, _f32p, _i32p, _f32p, ctypes.c_float, ctypes.c_float,
                                 ctypes.c_float, _f32p, _f32p, _i32p, _i32p, _i32p]
        l.ref_clue2d.restype = ctypes.c_int
        l.ref_clue2d_batch.argtypes = [ctypes.c_int32, _i64p, _f32p, _f32p, _i32p, _f32p, ctypes.c_float,
                                       ctypes.c_float, ctypes.c_float, _f32p, _f32p, _i32p, _i32p, _i32p,
                                       ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
        l.ref_clue2d_batch.restype = ctypes.c_int
        l.ref_clue3d.argtypes = ([ctypes.c_int32] + [_f32p] * 5 + [_i32p, _f32p, _i32p]
                                 + [ctypes.c_int32, ctypes.c_float, ctypes.c_float, ctypes.c_int32,
                                    ctypes.c_int32, ctypes.c_int32]
                                 + [ctypes.c_float] * 5
                                 + [_f32p, _f32p, _i32p, _i32p, _i32p, _i32p, _i32p, _i32p])
        l.ref_clue3d.restype = ctypes.c_int
        _ref = l
    return _ref


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _out2d(n):
    return dict(rho=np.empty(n, np.float32), delta=np.empty(n, np.float32),
                nearestHigher=np.empty(n, np.int32), isSeed=np.empty(n, np.int32),
                clusterIndex=np.empty(n, np.int32))


def _args2d(o):
    return (_p(o["rho"], _f32p), _p(o["delta"], _f32p), _p(o["nearestHigher"], _i32p),
            _p(o["isSeed"], _i32p), _p(o["clusterIndex"], _i32p))


def clue2d(x, y, layer, weight, dc, rhoc, odf):
    """One event through the CPU restatement.  Returns a dict of arrays."""
    x, y, w = _c(x, np.float32), _c(y, np.float32), _c(weight, np.float32)
    layer = _c(layer, np.int32)
    n = x.size
    o = _out2d(n)
    rc = lib().oracle_clue2d(n, _p(x, _f32p), _p(y, _f32p), _p(layer, _i32p), _p(w, _f32p), dc, rhoc, odf,
                             *_args2d(o))
    if rc:
        raise ValueError(f"oracle_clue2d failed ({rc})")
    return o


def clue2d_batch(offsets, x, y, layer, weight, dc, rhoc, odf, n_threads=1):
    """Concatenated events (CSR ``offsets``) over ``n_threads`` host threads."""
    offsets = _c(offsets, np.int64)
    x, y, w = _c(x, np.float32), _c(y, np.float32), _c(weight, np.float32)
    layer = _c(layer, np.int32)
    o = _out2d(x.size)
    rc = lib().oracle_clue2d_batch(offsets.size - 1, _p(offsets, _i64p), _p(x, _f32p), _p(y, _f32p),
                                   _p(layer, _i32p), _p(w, _f32p), dc, rhoc, odf, *_args2d(o), n_threads)
    if rc:
        raise ValueError(f"oracle_clue2d_batch failed ({rc})")
    return o


def ref_clue2d(x, y, layer, weight, dc, rhoc, odf):
    """One event through the unmodified reference (CLUEAlgoSerial::makeClusters)."""
    x, y, w = _c(x, np.float32), _c(y, np.float32), _c(weight, np.float32)
    layer = _c(layer, np.int32)
    n = x.size
    o = _out2d(n)
    ref_lib().ref_clue2d(n, _p(x, _f32p), _p(y, _f32p), _p(layer, _i32p), _p(w, _f32p), dc, rhoc, odf,
                         *_args2d(o))
    return o


def ref_clue2d_batch(offsets, x, y, layer, weight, dc, rhoc, odf, n_threads=1):
    """A CSR batch through the unmodified reference (CLUEAlgoSerial::makeClusters,
    one algorithm object per thread).  Returns (outputs dict, seconds spent in
    the makeClusters calls)."""
    offsets = _c(offsets, np.int64)
    x, y, w = _c(x, np.float32), _c(y, np.float32), _c(weight, np.float32)
    layer = _c(layer, np.int32)
    o = _out2d(x.size)
    sec = ctypes.c_double(0.0)
    ref_lib().ref_clue2d_batch(offsets.size - 1, _p(offsets, _i64p), _p(x, _f32p), _p(y, _f32p),
                               _p(layer, _i32p), _p(w, _f32p), dc, rhoc, odf, *_args2d(o), n_threads,
                               ctypes.byref(sec))
    return o, sec.value


def _out3d(n):
    return dict(rho=np.empty(n, np.float32), delta_t=np.empty(n, np.float32), delta_l=np.empty(n, np.int32),
                nh_layer=np.empty(n, np.int32), nh_idx=np.empty(n, np.int32), isSeed=np.empty(n, np.int32),
                tracksterIndex=np.empty(n, np.int32))


def _in3d(pts):
    f = {k: _c(pts[k], np.float32) for k in ("z", "eta", "phi", "r_over_absz", "radius", "energy")}
    i = {k: _c(pts[k], np.int32) for k in ("layer", "isSilicon")}
    return f, i


def clue3d(pts, **params):
    """One CLUE3D event through the CPU restatement.  ``pts`` maps the
    ClusterCollection field names to arrays; ``params`` override
    REFERENCE_3D_DEFAULTS.  Returns (outputs dict, n_tracksters)."""
    f, i = _in3d(pts)
    n = f["z"].size
    prm = Clue3DParams(**{**REFERENCE_3D_DEFAULTS, **params})
    o = _out3d(n)
    nt = lib().oracle_clue3d(n, _p(f["z"], _f32p), _p(f["eta"], _f32p), _p(f["phi"], _f32p),
                             _p(f["r_over_absz"], _f32p), _p(f["radius"], _f32p), _p(i["layer"], _i32p),
                             _p(f["energy"], _f32p), _p(i["isSilicon"], _i32p), ctypes.byref(prm),
                             _p(o["rho"], _f32p), _p(o["delta_t"], _f32p), _p(o["delta_l"], _i32p),
                             _p(o["nh_layer"], _i32p), _p(o["nh_idx"], _i32p), _p(o["isSeed"], _i32p),
                             _p(o["tracksterIndex"], _i32p))
    if nt < 0:
        raise ValueError(f"oracle_clue3d failed ({nt})")
    return o, nt


def clue3d_batch(offsets, pts, n_threads=1, **params):
    """CSR batch of CLUE3D events (``offsets``) through the CPU restatement
    over ``n_threads`` host threads.  Returns (outputs dict, per-event
    trackster counts)."""
    offsets = _c(offsets, np.int64)
    f, i = _in3d(pts)
    n = f["z"].size
    prm = Clue3DParams(**{**REFERENCE_3D_DEFAULTS, **params})
    o = _out3d(n)
    nts = np.zeros(offsets.size - 1, np.int32)
    rc = lib().oracle_clue3d_batch(offsets.size - 1, _p(offsets, _i64p), _p(f["z"], _f32p), _p(f["eta"], _f32p),
                                   _p(f["phi"], _f32p), _p(f["r_over_absz"], _f32p), _p(f["radius"], _f32p),
                                   _p(i["layer"], _i32p), _p(f["energy"], _f32p), _p(i["isSilicon"], _i32p),
                                   ctypes.byref(prm), _p(o["rho"], _f32p), _p(o["delta_t"], _f32p),
                                   _p(o["delta_l"], _i32p), _p(o["nh_layer"], _i32p), _p(o["nh_idx"], _i32p),
                                   _p(o["isSeed"], _i32p), _p(o["tracksterIndex"], _i32p), _p(nts, _i32p),
                                   n_threads)
    if rc:
        raise ValueError(f"oracle_clue3d_batch failed ({rc})")
    return o, nts


def ref_clue3d(pts, **params):
    """One CLUE3D event through the unmodified reference kernels (94 layers)."""
    f, i = _in3d(pts)
    n = f["z"].size
    p = {**REFERENCE_3D_DEFAULTS, **params}
    if p["n_layers"] != 94:
        raise ValueError("the reference tile geometry has 94 layers")
    o = _out3d(n)
    nt = ctypes.c_int32(0)
    ref_lib().ref_clue3d(n, _p(f["z"], _f32p), _p(f["eta"], _f32p), _p(f["phi"], _f32p),
                         _p(f["r_over_absz"], _f32p), _p(f["radius"], _f32p), _p(i["layer"], _i32p),
                         _p(f["energy"], _f32p), _p(i["isSilicon"], _i32p),
                         p["density_sibling_layers"], p["density_xy_distance_sqr"], p["kernel_density_factor"],
                         p["density_on_same_layer"], p["nh_sibling_layers"], p["nh_on_same_layer"],
                         p["critical_xy_distance"], p["critical_z_distance_lyr"], p["critical_density"],
                         p["critical_self_density"], p["outlier_multiplier"],
                         _p(o["rho"], _f32p), _p(o["delta_t"], _f32p), _p(o["delta_l"], _i32p),
                         _p(o["nh_layer"], _i32p), _p(o["nh_idx"], _i32p), _p(o["isSeed"], _i32p),
                         _p(o["tracksterIndex"], _i32p), ctypes.byref(nt))
    return o, nt.value
