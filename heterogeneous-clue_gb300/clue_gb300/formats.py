"""The reference's data formats around the clustering path.

* Inputs: the binary event files its Source module reads
  (src/serial/bin/Source.cc:8-80): ``raw2D`` (per event a uint32 point count
  then that many {float x, y, layer, weight} records), toy-detector files (one
  layer's {x, y, layer, weight} records with no header, replicated over the
  100 layers with layer += l), and ``raw3D`` (per event a uint32 count then
  40-byte {x, y, z, eta, phi, r_over_absz, radius, layer, energy, isSilicon}
  float records).  Layers (and isSilicon) are stored as floats and converted
  to int by truncation, as the reference's vector<int>::emplace_back does.
* Outputs: the per-event CSV of CLUEOutputProducer
  (src/serial/plugin-CLUEOutputProducer/CLUEOutputProducer.cc:38-45;
  header ``index,x,y,layer,weight,rho,delta,nh,isSeed,clusterId``, delta
  clamped at 999, default ostream formatting) and its file name
  (create_outputfileName, src/serial/DataFormats/CLUE_config.h:25-40).
* Validation: CLUEValidator's rules (src/serial/plugin-CLUEValidator/CLUEValidator.cc:42-89,135-195):
  floats within 1e-3, integers exact, delta clamped at 999, cluster ids equal
  up to a relabelling fixed by the seeds; results are only compared for the
  reference configuration dc=20, rhoc=25, odf=2.
"""
import numpy as np

from .synthetic import N_LAYERS

_POINT = np.dtype([("x", "<f4"), ("y", "<f4"), ("layer", "<f4"), ("weight", "<f4")])
_POINT_CLUS = np.dtype([(k, "<f4") for k in ("x", "y", "z", "eta", "phi", "r_over_absz", "radius", "layer",
                                              "energy", "isSilicon")])


def _to_int(a):
    # float -> int conversion of vector<int>::emplace_back(float): truncation toward zero
    return np.trunc(np.asarray(a, np.float32)).astype(np.int32)


def read_raw2d(path):
    """Events of a raw2D file as a list of dicts (x, y, layer, weight)."""
    buf = np.fromfile(path, dtype=np.uint8)
    events, pos = [], 0
    while pos + 4 <= buf.size:
        n = int(buf[pos:pos + 4].view("<u4")[0])
        pos += 4
        end = pos + n * _POINT.itemsize
        if end > buf.size:
            raise ValueError(f"{path}: truncated event ({n} points announced)")
        rec = buf[pos:end].view(_POINT)
        events.append(dict(x=rec["x"].copy(), y=rec["y"].copy(), layer=_to_int(rec["layer"]),
                           weight=rec["weight"].copy()))
        pos = end
    return events


def write_raw2d(path, events):
    with open(path, "wb") as f:
        for e in events:
            n = np.asarray(e["x"]).size
            rec = np.empty(n, _POINT)
            rec["x"], rec["y"], rec["weight"] = e["x"], e["y"], e["weight"]
            rec["layer"] = np.asarray(e["layer"], np.float32)
            f.write(np.uint32(n).tobytes())
            f.write(rec.tobytes())


def read_toy_detector(path, n_layers=N_LAYERS):
    """A toy-detector file: its records replicated over ``n_layers`` layers
    with layer += l (the reference's readToyDetectors)."""
    rec = np.fromfile(path, dtype=_POINT)
    reps = [dict(x=rec["x"], y=rec["y"], layer=_to_int(rec["layer"] + np.float32(l)), weight=rec["weight"])
            for l in range(n_layers)]
    return {k: np.concatenate([r[k] for r in reps]) for k in ("x", "y", "layer", "weight")}


def write_toy_detector(path, layer0):
    rec = np.empty(np.asarray(layer0["x"]).size, _POINT)
    for k in ("x", "y", "weight"):
        rec[k] = layer0[k]
    rec["layer"] = np.asarray(layer0["layer"], np.float32)
    rec.tofile(path)


def read_raw3d(path):
    """Events of a raw3D file as a list of ClusterCollection dicts."""
    buf = np.fromfile(path, dtype=np.uint8)
    events, pos = [], 0
    while pos + 4 <= buf.size:
        n = int(buf[pos:pos + 4].view("<u4")[0])
        pos += 4
        end = pos + n * _POINT_CLUS.itemsize
        if end > buf.size:
            raise ValueError(f"{path}: truncated event ({n} layer clusters announced)")
        rec = buf[pos:end].view(_POINT_CLUS)
        ev = {k: rec[k].copy() for k in _POINT_CLUS.names}
        ev["layer"] = _to_int(rec["layer"])
        ev["isSilicon"] = _to_int(rec["isSilicon"])
        events.append(ev)
        pos = end
    return events


def write_raw3d(path, events):
    with open(path, "wb") as f:
        for e in events:
            n = np.asarray(e["z"]).size
            rec = np.empty(n, _POINT_CLUS)
            for k in _POINT_CLUS.names:
                rec[k] = np.asarray(e.get(k, np.zeros(n)), np.float32)
            f.write(np.uint32(n).tobytes())
            f.write(rec.tobytes())


def source_2d(path, max_events=-1):
    """The event stream of the reference's Source2D (src/serial/bin/Source.cc:88-118,
    147-186): a path containing "toyDetector" is one replicated cloud, replayed
    10 times by default; any other file is raw2D, one cloud per event, each
    once by default.  Events cycle through the clouds; ids start at 1.
    Yields (event id, cloud)."""
    toy = "toyDetector" in str(path)
    clouds = [read_toy_detector(path)] if toy else read_raw2d(path)
    n = max_events if max_events >= 0 else (10 if toy else len(clouds))
    for i in range(n if clouds else 0):
        yield i + 1, clouds[i % len(clouds)]


def source_3d(path, max_events=-1):
    """Source3D's stream (Source.cc:124-143,190-226): raw3D events, each once by
    default, cycled; ids start at 1.  Yields (event id, ClusterCollection dict)."""
    clouds = read_raw3d(path)
    n = max_events if max_events >= 0 else len(clouds)
    for i in range(n if clouds else 0):
        yield i + 1, clouds[i % len(clouds)]


def read_config(path):
    """A parameter file ``dc,rhoc,outlierDeltaFactor,produceOutput`` (one
    line, as config/hgcal_config.csv; parsed like src/serial/bin/main.cc:131-140:
    three floats, then an int read as a bool).  Returns (dc, rhoc, odf, produce_output)."""
    with open(path) as f:
        fields = f.read().strip().split(",")
    if len(fields) != 4:
        raise ValueError(f"{path}: expected dc,rhoc,outlierDeltaFactor,produceOutput")
    return (float(np.float32(fields[0])), float(np.float32(fields[1])), float(np.float32(fields[2])),
            bool(int(fields[3])))


def output_file_name(event_id, dc, rhoc, odf):
    """create_outputfileName: Event_<id>_<dc>_<rhoc>_<odf>.csv, two decimals."""
    return f"Event_{int(event_id)}_{dc:.2f}_{rhoc:.2f}_{odf:.2f}.csv"


def _g(v):
    # std::ostream default float formatting: 6 significant digits, like %g
    return f"{float(v):g}"


def write_output_csv(path, event, out):
    """CLUEOutputProducer's CSV of one event and its outputs."""
    x, y, l, w = event["x"], event["y"], event["layer"], event["weight"]
    rho, delta = out["rho"], out["delta"]
    nh, seed, ci = out["nearestHigher"], out["isSeed"], out["clusterIndex"]
    with open(path, "w") as f:
        f.write("index,x,y,layer,weight,rho,delta,nh,isSeed,clusterId\n")
        for i in range(len(x)):
            d = 999.0 if delta[i] > 999 else delta[i]
            f.write(f"{i},{_g(x[i])},{_g(y[i])},{int(l[i])},{_g(w[i])},{_g(rho[i])},{_g(d)},"
                    f"{int(nh[i])},{int(seed[i])},{int(ci[i])}\n")


def read_output_csv(path):
    """The columns of an output CSV (the reference golden files have this layout)."""
    a = np.loadtxt(path, delimiter=",", skiprows=1, ndmin=2)
    cols = {}
    names = ("index", "x", "y", "layer", "weight", "rho", "delta", "nh", "isSeed", "clusterId")
    for j, k in enumerate(names):
        cols[k] = a[:, j]
    return dict(x=cols["x"].astype(np.float32), y=cols["y"].astype(np.float32), layer=cols["layer"].astype(np.int32),
                weight=cols["weight"].astype(np.float32), rho=cols["rho"].astype(np.float32),
                delta=cols["delta"].astype(np.float32), nearestHigher=cols["nh"].astype(np.int32),
                isSeed=cols["isSeed"].astype(np.int32), clusterIndex=cols["clusterId"].astype(np.int32))


def _close(a, b, tol=1e-3):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return a.shape == b.shape and bool(np.all(np.abs(a - b) <= tol))


def clusters_equal(got, truth):
    """CLUEValidator::arraysClustersEqual: ids compared through the map
    seed's id -> true id; -1 stays -1."""
    ci, seed, tci = np.asarray(got["clusterIndex"]), np.asarray(got["isSeed"]), np.asarray(truth["clusterIndex"])
    mapping = {}
    for i in np.flatnonzero(seed):
        mapping[int(ci[i])] = int(tci[i])
    for i in range(ci.size):
        m = -1 if ci[i] == -1 else mapping.get(int(ci[i]), 0)
        if m != tci[i]:
            return False
    return True


def validate(event, out, truth, params):
    """CLUEValidator::validateOutput.  Returns (ok, messages)."""
    msgs, ok = [], True
    for k in ("x", "y", "weight"):
        if not _close(event[k], truth[k]):
            return False, [f"input {k} differs"]
    if not np.array_equal(np.asarray(event["layer"]), truth["layer"]):
        return False, ["input layer differs"]
    msgs.append("input variables are correct")
    dc, rhoc, odf = params
    if (np.float32(dc), np.float32(rhoc), np.float32(odf)) != (np.float32(20), np.float32(25), np.float32(2)):
        msgs.append("parameters differ from the reference files' (20, 25, 2): results not checked")
        return True, msgs
    checks = [("rho", _close(out["rho"], truth["rho"])),
              ("delta", _close(np.minimum(np.asarray(out["delta"], np.float32), 999), truth["delta"])),
              ("nearestHigher", np.array_equal(out["nearestHigher"], truth["nearestHigher"])),
              ("isSeed", np.array_equal(out["isSeed"], truth["isSeed"])),
              ("cluster ids", clusters_equal(out, truth))]
    for name, good in checks:
        msgs.append(f"output {name} -> {'ok' if good else 'FAILED'}")
        ok &= good
    return ok, msgs
