"""The reference's input/output formats and validator rules (host code),
plus one GPU round trip: a raw2D file replayed through the CUDA path and
validated against the oracle's CSV the way the reference's validator does."""
import numpy as np
import pytest

import clue_gb300 as C
import oracle
from clue_gb300 import formats as F
from clue_gb300 import synthetic as S

from _util import assert_bitexact

REF = (20.0, 25.0, 2.0)


def test_raw2d_round_trip(tmp_path):
    b = S.uneven_batch(3, seed=2, lo=1000, hi=4000)
    evs = [S.event_of(b, e) for e in range(3)]
    p = tmp_path / "events.bin"
    F.write_raw2d(p, evs)
    back = F.read_raw2d(p)
    assert len(back) == 3
    for a, e in zip(back, evs):
        for k in ("x", "y", "weight", "layer"):
            assert np.array_equal(a[k], e[k]), k


def test_raw2d_truncated_file_is_an_error(tmp_path):
    p = tmp_path / "bad.bin"
    F.write_raw2d(p, [S.toy_event(1, blobs_per_layer=1, noise_per_layer=1)])
    data = p.read_bytes()
    p.write_bytes(data[:-5])
    with pytest.raises(ValueError):
        F.read_raw2d(p)


def test_toy_detector_replicates_one_layer(tmp_path):
    ev = S.toy_event(3, blobs_per_layer=2, noise_per_layer=10)
    layer0 = {k: v[ev["layer"] == 0] for k, v in ev.items()}
    p = tmp_path / "toyDetector_test.bin"
    F.write_toy_detector(p, layer0)
    full = F.read_toy_detector(p)
    n0 = layer0["x"].size
    assert full["x"].size == 100 * n0
    assert np.array_equal(full["layer"][:n0], np.zeros(n0, np.int32))
    assert np.array_equal(full["layer"][-n0:], np.full(n0, 99, np.int32))
    assert np.array_equal(full["x"][5 * n0:6 * n0], layer0["x"])


def test_raw3d_round_trip(tmp_path):
    evs = [S.clue3d_event(s, n_clusters=300, n_layers=94) for s in (1, 2)]
    p = tmp_path / "raw3D.bin"
    F.write_raw3d(p, evs)
    back = F.read_raw3d(p)
    for a, e in zip(back, evs):
        for k in ("z", "eta", "phi", "r_over_absz", "radius", "energy"):
            assert np.array_equal(a[k], e[k]), k
        assert np.array_equal(a["layer"], e["layer"]) and np.array_equal(a["isSilicon"], e["isSilicon"])


def test_source_streams(tmp_path):
    ev = S.toy_event(3, blobs_per_layer=1, noise_per_layer=3)
    layer0 = {k: v[ev["layer"] == 0] for k, v in ev.items()}
    toy = tmp_path / "toyDetector_1k.bin"
    F.write_toy_detector(toy, layer0)
    got = list(F.source_2d(toy))
    assert [i for i, _ in got] == list(range(1, 11))  # ten replays of the one cloud by default
    assert got[0][1]["x"].size == 100 * layer0["x"].size
    assert len(list(F.source_2d(toy, max_events=3))) == 3
    b = S.uneven_batch(3, seed=4, lo=1000, hi=2000)
    raw = tmp_path / "raw2D.bin"
    F.write_raw2d(raw, [S.event_of(b, e) for e in range(3)])
    ids = [(i, c["x"].size) for i, c in F.source_2d(raw, max_events=5)]
    sizes = [int(b["offsets"][e + 1] - b["offsets"][e]) for e in range(3)]
    assert ids == [(1, sizes[0]), (2, sizes[1]), (3, sizes[2]), (4, sizes[0]), (5, sizes[1])]
    r3 = tmp_path / "raw3D.bin"
    F.write_raw3d(r3, [S.clue3d_event(1, n_clusters=50)])
    assert [i for i, _ in F.source_3d(r3, max_events=2)] == [1, 2]


def test_config_files(tmp_path):
    p = tmp_path / "hgcal_config.csv"
    p.write_text("1.3,0.11,2,0")
    assert F.read_config(p) == (float(np.float32(1.3)), float(np.float32(0.11)), 2.0, False)
    p.write_text("20,25,2,1\n")
    assert F.read_config(p) == (20.0, 25.0, 2.0, True)
    p.write_text("20,25\n")
    with pytest.raises(ValueError):
        F.read_config(p)


def test_output_csv_and_validator(tmp_path):
    ev = S.toy_event(777, blobs_per_layer=4, noise_per_layer=40)
    out = oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *REF)
    assert F.output_file_name(3, *REF) == "Event_3_20.00_25.00_2.00.csv"
    p = tmp_path / F.output_file_name(0, *REF)
    F.write_output_csv(p, ev, out)
    truth = F.read_output_csv(p)
    assert open(p).readline().strip() == "index,x,y,layer,weight,rho,delta,nh,isSeed,clusterId"
    ok, msgs = F.validate(ev, out, truth, REF)
    assert ok, msgs
    # cluster ids relabelled consistently still validate
    perm = np.random.default_rng(0).permutation(int(out["clusterIndex"].max()) + 1)
    rel = dict(out)
    rel["clusterIndex"] = np.where(out["clusterIndex"] >= 0, perm[np.maximum(out["clusterIndex"], 0)], -1)
    assert F.validate(ev, rel, truth, REF)[0]
    # a moved label and a perturbed rho are caught
    bad = dict(out)
    bad["clusterIndex"] = out["clusterIndex"].copy()
    i = int(np.flatnonzero(out["isSeed"] == 0)[0])
    bad["clusterIndex"][i] = (bad["clusterIndex"][i] + 1) % (int(out["clusterIndex"].max()) + 1)
    assert not F.validate(ev, bad, truth, REF)[0]
    bad2 = dict(out)
    bad2["rho"] = out["rho"] + np.float32(0.01)
    assert not F.validate(ev, bad2, truth, REF)[0]
    # other parameters: inputs checked, results not
    ok, msgs = F.validate(ev, out, truth, (1.3, 2.0, 2.0))
    assert ok and "not checked" in msgs[-1]


@pytest.mark.gpu
def test_raw2d_replayed_through_cuda_validates(tmp_path, cuda_lib):
    evs = [S.toy_event(s, blobs_per_layer=6, noise_per_layer=60) for s in (10, 11)]
    p = tmp_path / "raw2D.bin"
    F.write_raw2d(p, evs)
    algo = C.Clusterizer(*REF)
    for k, ev in enumerate(F.read_raw2d(p)):
        got = algo.make_clusters(ev["x"], ev["y"], ev["layer"], ev["weight"])
        want = oracle.clue2d(ev["x"], ev["y"], ev["layer"], ev["weight"], *REF)
        assert_bitexact(got, want)
        csv = tmp_path / F.output_file_name(k, *REF)
        F.write_output_csv(csv, ev, want)
        ok, msgs = F.validate(ev, got, F.read_output_csv(csv), REF)
        assert ok, msgs
    algo.close()
