"""Seeded synthetic HGCAL-like events.

The reference benchmarks on toy-detector and HGCAL files that it downloads at
build time (data/url.txt); none is available here, so events are generated
with the same shapes: 100 layers, Gaussian blobs of hits on a uniform noise
floor inside the [-250, 250] cm tile domain.  Within an event, points come
out layer by layer (blob points, then noise, for layer 0, then layer 1, ...),
as the reference's toy-detector reader lays them out
(src/serial/bin/Source.cc:62-80); ``shuffle=True`` permutes each event.

All arrays are float32 x, y, weight and int32 layer, the PointsCloud layout
(src/serial/DataFormats/PointsCloud.h:6-13); batches are CSR (``offsets``).
The generator is vectorised over events and layers: a whole batch is a
handful of numpy calls.
"""
import math

import numpy as np

N_LAYERS = 100


def _batch(rng, blobs_per_layer, noise_per_layer, size_fn, sigma_fn, shuffle=False):
    """Events e = 0..E-1 with ``blobs_per_layer[e]`` Gaussian blobs per layer
    (centre U[-200,200]^2, sizes ``size_fn(rng, k)``, sigma ``sigma_fn(rng, k)``,
    weights LogNormal(0, 0.5)) and ``noise_per_layer[e]`` uniform noise points
    per layer in [-250,250]^2 (weights Exp(mean 0.1))."""
    nb = np.asarray(blobs_per_layer, np.int64)
    nn = np.asarray(noise_per_layer, np.int64)
    E = nb.size
    G = E * N_LAYERS                                  # (event, layer) groups
    blobs_in_group = np.repeat(nb, N_LAYERS)          # [G]
    B = int(blobs_in_group.sum())
    sizes = np.asarray(size_fn(rng, B), np.int64)
    cx = rng.uniform(-200.0, 200.0, B).astype(np.float32)
    cy = rng.uniform(-200.0, 200.0, B).astype(np.float32)
    sg = np.asarray(sigma_fn(rng, B), np.float32)
    M = int(sizes.sum())
    bx = np.repeat(cx, sizes) + rng.standard_normal(M, dtype=np.float32) * np.repeat(sg, sizes)
    by = np.repeat(cy, sizes) + rng.standard_normal(M, dtype=np.float32) * np.repeat(sg, sizes)
    bw = np.exp(np.float32(0.5) * rng.standard_normal(M, dtype=np.float32)).astype(np.float32)
    noise_in_group = np.repeat(nn, N_LAYERS)          # [G]
    K = int(noise_in_group.sum())
    nx = rng.uniform(-250.0, 250.0, K).astype(np.float32)
    ny = rng.uniform(-250.0, 250.0, K).astype(np.float32)
    nw = (np.float32(0.1) * rng.standard_exponential(K, dtype=np.float32)).astype(np.float32)

    group_of_blob = np.repeat(np.arange(G), blobs_in_group)
    blob_pts_in_group = np.bincount(group_of_blob, weights=sizes, minlength=G).astype(np.int64)
    per_group = blob_pts_in_group + noise_in_group
    gstart = np.zeros(G + 1, np.int64)
    np.cumsum(per_group, out=gstart[1:])
    # blob points: group start + rank among the group's blob points
    group_of_bpt = np.repeat(group_of_blob, sizes)
    first_bpt = np.zeros(G + 1, np.int64)
    np.cumsum(blob_pts_in_group, out=first_bpt[1:])
    pos_b = gstart[group_of_bpt] + (np.arange(M) - first_bpt[group_of_bpt])
    # noise points: after the group's blob points
    group_of_npt = np.repeat(np.arange(G), noise_in_group)
    first_npt = np.zeros(G + 1, np.int64)
    np.cumsum(noise_in_group, out=first_npt[1:])
    pos_n = gstart[group_of_npt] + blob_pts_in_group[group_of_npt] + (np.arange(K) - first_npt[group_of_npt])

    n = M + K
    x = np.empty(n, np.float32)
    y = np.empty(n, np.float32)
    w = np.empty(n, np.float32)
    l = np.empty(n, np.int32)
    x[pos_b], y[pos_b], w[pos_b] = bx, by, bw
    x[pos_n], y[pos_n], w[pos_n] = nx, ny, nw
    l[pos_b] = (group_of_bpt % N_LAYERS).astype(np.int32)
    l[pos_n] = (group_of_npt % N_LAYERS).astype(np.int32)
    offsets = gstart[::N_LAYERS].copy()
    if shuffle:
        for e in range(E):
            s, t = offsets[e], offsets[e + 1]
            p = s + rng.permutation(t - s)
            x[s:t], y[s:t], w[s:t], l[s:t] = x[p], y[p], w[p], l[p]
    return dict(offsets=offsets, x=x, y=y, layer=l, weight=w)


def event_of(batch, e):
    """Event ``e`` of a CSR batch as a dict of array views."""
    s, t = batch["offsets"][e], batch["offsets"][e + 1]
    return {k: batch[k][s:t] for k in ("x", "y", "layer", "weight")}


def toy_event(seed=12345, blobs_per_layer=20, blob_size=40, noise_per_layer=200, shuffle=False):
    """Toy-detector event: 100 layers x (20 blobs x 40 points at sigma 1 cm
    + 200 noise points) = 100,000 points."""
    rng = np.random.default_rng(seed)
    b = _batch(rng, [blobs_per_layer], [noise_per_layer], lambda r, k: np.full(k, blob_size, np.int64),
               lambda r, k: np.ones(k, np.float32), shuffle)
    return event_of(b, 0)


def _hgcal_size(r, k):
    return r.integers(30, 81, k)


def _hgcal_sigma(r, k):
    return r.uniform(0.7, 1.5, k).astype(np.float32)


def hgcal_batch(n_events, seed=1000, blobs_per_layer=50, noise_per_layer=500, shuffle=False):
    """HGCAL-occupancy events: 100 layers x (50 blobs of U{30..80} points at
    sigma U[0.7, 1.5] cm + 500 noise points), about 325k points each."""
    rng = np.random.default_rng(seed)
    return _batch(rng, [blobs_per_layer] * n_events, [noise_per_layer] * n_events, _hgcal_size, _hgcal_sigma,
                  shuffle)


def hgcal_event(seed=1000, **kw):
    return event_of(hgcal_batch(1, seed, **kw), 0)


def uneven_sizes(n_events, seed=7, lo=5000, hi=200000):
    """Per-event hit counts drawn log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(math.log(lo), math.log(hi), n_events)
    return np.rint(np.exp(u)).astype(np.int64)


def uneven_batch(n_events, seed=7, lo=5000, hi=200000, shuffle=False):
    """The batched workload: ``n_events`` events whose target sizes are
    log-uniform in [lo, hi]; each is generated with 15 % noise and
    round((N/100 - noise)/55) blobs of U{30..80} points per layer."""
    sizes = uneven_sizes(n_events, seed, lo, hi)
    per_layer = sizes / N_LAYERS
    noise = np.rint(0.15 * per_layer).astype(np.int64)
    blobs = np.maximum(np.rint((per_layer - noise) / 55.0).astype(np.int64), 0)
    rng = np.random.default_rng(seed + 1)
    return _batch(rng, blobs, noise, _hgcal_size, _hgcal_sigma, shuffle)


# ----------------------------------------------------------------------------
# CLUE3D layer clusters
# ----------------------------------------------------------------------------

CLUE3D_FIELDS = ("x", "y", "z", "eta", "phi", "r_over_absz", "radius", "layer", "energy", "isSilicon")


def layer_z(n_layers=N_LAYERS):
    """HGCAL-like layer positions, 320..520 cm."""
    return (320.0 + 200.0 * np.arange(n_layers) / max(n_layers - 1, 1)).astype(np.float32)


def clue3d_event(seed, n_clusters=None, n_layers=N_LAYERS, radius=2.0, eta_range=(1.5, 3.0)):
    """Layer clusters for CLUE3D: eta U[1.5, 3.0], phi U[-pi, pi], energy
    LogNormal(0, 0.7), layer U{0..n_layers-1}.  The fields the reference
    also consumes are derived: z from the layer table, r/|z| = 1/sinh(eta),
    isSilicon = 1, radius fixed."""
    rng = np.random.default_rng(seed)
    k = int(n_clusters) if n_clusters is not None else int(rng.integers(2000, 20001))
    eta = rng.uniform(eta_range[0], eta_range[1], k).astype(np.float32)
    phi = rng.uniform(-math.pi, math.pi, k).astype(np.float32)
    energy = np.exp(0.7 * rng.standard_normal(k)).astype(np.float32)
    layer = rng.integers(0, n_layers, k).astype(np.int32)
    z = layer_z(n_layers)[layer]
    roa = (1.0 / np.sinh(eta.astype(np.float64))).astype(np.float32)
    r = roa * z
    return dict(x=(r * np.cos(phi)).astype(np.float32), y=(r * np.sin(phi)).astype(np.float32),
                z=z.astype(np.float32), eta=eta, phi=phi, r_over_absz=roa,
                radius=np.full(k, radius, np.float32), layer=layer, energy=energy,
                isSilicon=np.ones(k, np.int32))


def concat3d(events):
    sizes = np.array([e["z"].size for e in events], np.int64)
    off = np.zeros(len(events) + 1, np.int64)
    np.cumsum(sizes, out=off[1:])
    out = {k: np.concatenate([e[k] for e in events]) for k in CLUE3D_FIELDS}
    out["offsets"] = off
    return out


def clue3d_batch(n_events, seed0=1000, n_layers=N_LAYERS, **kw):
    """``n_events`` CLUE3D events, event e from seed seed0 + e."""
    return concat3d([clue3d_event(seed0 + e, n_layers=n_layers, **kw) for e in range(n_events)])


def event3d_of(batch, e):
    s, t = batch["offsets"][e], batch["offsets"][e + 1]
    return {k: batch[k][s:t] for k in CLUE3D_FIELDS}
