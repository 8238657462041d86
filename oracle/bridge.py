"""CPU statement of the 2D -> 3D bridge (test infrastructure, not product code).

The bridge has no reference counterpart (the reference's CLUE3D reads raw3D
files, src/serial/bin/Source.cc:43-60), so this module is its definition
rather than a restatement; parity with it is "defined here", not pinned to the
reference.  Layer cluster c of event e = the 2D points with clusterIndex c
(clusters of an event in id order); sums are exact fixed-point integers
(weights x 2^24, weight * coordinate x 2^16, each rounded to nearest even),
so accumulation order does not matter; x, y = (S_wx * 2^8) / S_w in double,
rounded to float; layer = the seed's; z = layer_z[layer]; r = |(x, y)| in
double; r_over_absz = r / |z|; eta = asinh(z / max(r, 1e-9)); phi = atan2(y, x);
clusters with zero total weight take the seed's position.
"""
import numpy as np


def layer_clusters(offsets, x, y, layer, weight, isSeed, clusterIndex, layer_z, radius=2.0, is_silicon=1):
    """Returns (cluster_offsets, dict of the ClusterCollection fields)."""
    offsets = np.asarray(offsets, np.int64)
    E = offsets.size - 1
    ev = np.repeat(np.arange(E), np.diff(offsets))
    seed = np.asarray(isSeed) != 0
    counts = np.bincount(ev[seed], minlength=E).astype(np.int64)
    coff = np.zeros(E + 1, np.int64)
    np.cumsum(counts, out=coff[1:])
    C = int(coff[-1])
    ci = np.asarray(clusterIndex)
    m = ci >= 0
    g = coff[ev[m]] + ci[m]
    wd = np.asarray(weight, np.float32)[m].astype(np.float64)
    xd = np.asarray(x, np.float32)[m].astype(np.float64)
    yd = np.asarray(y, np.float32)[m].astype(np.float64)
    sw = np.zeros(C, np.int64)
    swx = np.zeros(C, np.int64)
    swy = np.zeros(C, np.int64)
    np.add.at(sw, g, np.rint(wd * 2.0 ** 24).astype(np.int64))
    np.add.at(swx, g, np.rint(wd * xd * 2.0 ** 16).astype(np.int64))
    np.add.at(swy, g, np.rint(wd * yd * 2.0 ** 16).astype(np.int64))
    seed_of = np.zeros(C, np.int64)
    gs = coff[ev[seed]] + ci[seed]
    seed_of[gs] = np.flatnonzero(seed)
    L = np.asarray(layer, np.int32)[seed_of]
    nz = sw != 0
    den = np.where(nz, sw, 1).astype(np.float64)
    xb = np.where(nz, (swx.astype(np.float64) * 256.0 / den).astype(np.float32), np.asarray(x, np.float32)[seed_of])
    yb = np.where(nz, (swy.astype(np.float64) * 256.0 / den).astype(np.float32), np.asarray(y, np.float32)[seed_of])
    z = np.asarray(layer_z, np.float32)[L]
    r = np.sqrt(xb.astype(np.float64) ** 2 + yb.astype(np.float64) ** 2)
    out = dict(x=xb, y=yb, z=z,
               eta=np.arcsinh(z.astype(np.float64) / np.maximum(r, 1e-9)).astype(np.float32),
               phi=np.arctan2(yb.astype(np.float64), xb.astype(np.float64)).astype(np.float32),
               r_over_absz=(r / np.abs(z.astype(np.float64))).astype(np.float32),
               radius=np.full(C, radius, np.float32), layer=L.astype(np.int32),
               energy=(sw.astype(np.float64) / 2.0 ** 24).astype(np.float32),
               isSilicon=np.full(C, is_silicon, np.int32))
    return coff, out
