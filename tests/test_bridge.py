"""2D -> 3D bridge: layer clusters built on the device from a clustered 2D
batch and fed to CLUE3D without the point data leaving the device.

The bridge has no reference counterpart; oracle/bridge.py states its
definition.  Tolerances: every field is bit-exact except eta and phi, which
come from double asinh/atan2 whose last bits may differ between the CPU and
CUDA math libraries before rounding to float: those are allowed 1 float ulp.
The CLUE3D stage after the bridge is bit-exact against the oracle run on the
bridge's own (GPU) output."""
import numpy as np
import pytest

import clue_gb300 as C
import oracle
from oracle import bridge as OB
from clue_gb300 import synthetic as S

from _util import KEYS_3D, assert_bitexact, max_ulp

PRM2D = (1.3, 2.0, 2.0)
EXACT = ("x", "y", "z", "r_over_absz", "radius", "layer", "energy", "isSilicon")


def _batch_with_outputs(n_events, seed):
    b = S.uneven_batch(n_events, seed=seed, lo=2000, hi=40000)
    o = oracle.clue2d_batch(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], *PRM2D, n_threads=4)
    return b, o


def test_bridge_definition_properties():
    b, o = _batch_with_outputs(3, 5)
    coff, lc = OB.layer_clusters(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], o["isSeed"],
                                 o["clusterIndex"], S.layer_z())
    ev = np.repeat(np.arange(3), np.diff(b["offsets"]))
    assert np.array_equal(np.diff(coff), np.bincount(ev[o["isSeed"] != 0], minlength=3))
    for e in range(3):
        s, t = b["offsets"][e], b["offsets"][e + 1]
        ci, w = o["clusterIndex"][s:t], b["weight"][s:t]
        m = ci >= 0
        # energies add up to the clustered weight, to fixed-point rounding
        tot = lc["energy"][coff[e]:coff[e + 1]].astype(np.float64).sum()
        assert abs(tot - w[m].astype(np.float64).sum()) < 1e-3 * max(1.0, tot)
        # every 2D cluster lies in one layer: the layer cluster's
        for c in range(0, int(coff[e + 1] - coff[e]), 97):
            lay = b["layer"][s:t][ci == c]
            assert np.all(lay == lc["layer"][coff[e] + c])
            xs = b["x"][s:t][ci == c]
            assert xs.min() - 1e-3 <= lc["x"][coff[e] + c] <= xs.max() + 1e-3


def _compare(got, want):
    for k in EXACT:
        g, w = np.asarray(got[k]), np.asarray(want[k])
        assert g.dtype == w.dtype and np.array_equal(g.view(np.int32), w.view(np.int32)), k
    for k in ("eta", "phi"):
        assert max_ulp(got[k], want[k]) <= 1, k


@pytest.mark.gpu
def test_bridge_then_clue3d_on_device(cuda_lib):
    import torch
    b, _ = _batch_with_outputs(6, 17)
    n = int(b["offsets"][-1])
    d = {k: torch.from_numpy(np.ascontiguousarray(b[k])).cuda() for k in ("x", "y", "layer", "weight")}
    out2d = {k: torch.empty(n, dtype=torch.float32 if k in ("rho", "delta") else torch.int32, device="cuda")
             for k in ("rho", "delta", "nearestHigher", "isSeed", "clusterIndex")}
    algo = C.Clusterizer(*PRM2D)
    algo.run_batch(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], out=out2d, flags=C.DEVICE_MEMORY)
    algo.synchronize()
    h2d = {k: v.cpu().numpy() for k, v in out2d.items()}
    coff, lc = algo.layer_clusters(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], out2d)
    wcoff, want = OB.layer_clusters(b["offsets"], b["x"], b["y"], b["layer"], b["weight"], h2d["isSeed"],
                                    h2d["clusterIndex"], S.layer_z())
    assert np.array_equal(coff, wcoff)
    got = {k: v.cpu().numpy() for k, v in lc.items()}
    _compare(got, want)
    # deterministic: a second build gives the same bits
    _, lc2 = algo.layer_clusters(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], out2d)
    for k in got:
        assert np.array_equal(lc2[k].cpu().numpy().view(np.int32), got[k].view(np.int32)), k
    # CLUE3D straight from the device-resident layer clusters
    prm3 = dict(n_layers=100)
    C3 = int(coff[-1])
    out3 = {k: torch.empty(C3, dtype=torch.float32 if k in ("rho", "delta_transverse") else torch.int32,
                           device="cuda")
            for k in ("rho", "delta_transverse", "delta_layers", "nh_layer", "nh_index", "isSeed", "tracksterIndex")}
    _, nts = algo.run_clue3d(coff, lc, params=prm3, flags=C.DEVICE_MEMORY, out=out3)
    algo.synchronize()
    names = dict(rho="rho", delta_transverse="delta_t", delta_layers="delta_l", nh_layer="nh_layer",
                 nh_index="nh_idx", isSeed="isSeed", tracksterIndex="tracksterIndex")
    g3 = {names[k]: v.cpu().numpy() for k, v in out3.items()}
    for e in range(coff.size - 1):
        s, t = coff[e], coff[e + 1]
        w3, _ = oracle.clue3d({k: got[k][s:t] for k in got}, **prm3)
        assert_bitexact({k: v[s:t] for k, v in g3.items()}, w3, KEYS_3D, label=f"event {e}")
    algo.close()


@pytest.mark.gpu
def test_bridge_errors(cuda_lib):
    import torch
    b, o = _batch_with_outputs(2, 3)
    n = int(b["offsets"][-1])
    d = {k: torch.from_numpy(np.ascontiguousarray(b[k])).cuda() for k in ("x", "y", "layer", "weight")}
    o2 = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in o.items()}
    algo = C.Clusterizer(*PRM2D)
    with pytest.raises(C.ClueError, match="layer"):  # z table shorter than the layers used
        algo.layer_clusters(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], o2, layer_z=S.layer_z(10))
    bad = dict(o2)
    ci = o["clusterIndex"].copy()
    ci[np.flatnonzero(ci >= 0)[0]] = 10 ** 6
    bad["clusterIndex"] = torch.from_numpy(ci).cuda()
    with pytest.raises(C.ClueError, match="clusterIndex"):
        algo.layer_clusters(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], bad)
    # the handle stays usable
    coff, lc = algo.layer_clusters(b["offsets"], d["x"], d["y"], d["layer"], d["weight"], o2)
    assert int(coff[-1]) == int((o["isSeed"] != 0).sum())
    assert n > 0
    algo.close()
