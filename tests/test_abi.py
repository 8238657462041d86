"""CPU-side checks of the drop-in boundary: the library loads, exports every
entry point include/clue.h declares, and reports errors through codes and
messages (no GPU is needed for any of this)."""
import ctypes
import os
import subprocess

import pytest

import clue_gb300 as C

from conftest import ROOT, gpu_available


def test_library_exports_every_declared_symbol(cuda_lib):
    declared = C.header_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(cuda_lib, s)]
    assert not missing, f"declared in include/clue.h but not exported: {missing}"


def test_entry_points_have_c_linkage():
    # plain (unmangled) text symbols: what cgo / JNI / ctypes / a C++ plugin bind to
    out = subprocess.run(["nm", "-D", "--defined-only", C.LIB_PATH], capture_output=True, text=True).stdout
    for name in C.header_symbols():
        assert f" T {name}\n" in out + "\n", name


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_create_without_gpu_reports_cuda_error(cuda_lib):
    h = ctypes.c_void_p()
    rc = cuda_lib.clue_create(ctypes.byref(C.Params(1.3, 2.0, 2.0)), 0, 0, None, ctypes.byref(h))
    assert rc == C.CLUE_ECUDA
    assert C.last_error()
    assert not h


def test_null_arguments_are_einval(cuda_lib):
    assert cuda_lib.clue_create(None, 0, 0, None, None) == C.CLUE_EINVAL
    assert cuda_lib.clue_run_event(None, 0, None, None, None, None, None, 0) == C.CLUE_EINVAL
    assert cuda_lib.clue_run_batch(None, 0, None, None, None, None, None, None, 0) == C.CLUE_EINVAL
    assert "NULL" in C.last_error()
    assert cuda_lib.clue_destroy(None) == C.CLUE_OK
    assert cuda_lib.clue_set_stream(None, None) == C.CLUE_EINVAL
    assert cuda_lib.clue_last_run_stats(None, None) == C.CLUE_EINVAL
    assert cuda_lib.clue_bridge_count(None, 0, None, None, None) == C.CLUE_EINVAL
    assert cuda_lib.clue_bridge_build(None, None, 0, None, None, None, None, None, None, None, None, None) == \
        C.CLUE_EINVAL
    assert cuda_lib.clue_server_submit_many(None, 0, None, None, None, None, None, None, None) == C.CLUE_EINVAL
    assert cuda_lib.clue_server_poll(None, 0, 0, None) == C.CLUE_EINVAL
    assert cuda_lib.clue3d_run_batch(None, None, 0, None, None, None, None, 0) == C.CLUE_EINVAL
    assert cuda_lib.clue_run_event_noalloc(None, 1, None, None, None, None, None, None) == C.CLUE_EINVAL
    assert cuda_lib.clue_run_event_noalloc(None, -1, None, None, None, None, None, None) == C.CLUE_EINVAL


def test_noalloc_warm_up_without_gpu_reports_cuda_error(cuda_lib):
    """The n = 0 warm-up call needs a device for its set-up; here there is none."""
    assert cuda_lib.clue_run_event_noalloc(None, 0, None, None, None, None, None, None) == C.CLUE_ECUDA
    assert C.last_error()


def test_required_bytes_grows_with_points(cuda_lib):
    a = cuda_lib.clue_required_bytes(1, 100_000, C.DEVICE_MEMORY)
    b = cuda_lib.clue_required_bytes(1, 200_000, C.DEVICE_MEMORY)
    c = cuda_lib.clue_required_bytes(1, 200_000, C.HOST_MEMORY)
    assert 0 < a < b < c
    assert cuda_lib.clue_required_bytes(-1, 10, 0) == 0


def test_default_params3d_are_the_reference_defaults(cuda_lib):
    p = C.default_params3d()
    assert (p.n_layers, p.density_sibling_layers, p.nh_sibling_layers) == (94, 3, 3)
    assert abs(p.density_xy_distance_sqr - 3.24) < 1e-6 and abs(p.kernel_density_factor - 0.2) < 1e-7
    assert (p.critical_xy_distance, p.critical_z_distance_lyr) == (pytest.approx(1.8), 5.0)
    assert (p.critical_density, p.critical_self_density, p.outlier_multiplier) == (
        pytest.approx(0.6), pytest.approx(0.15), 2.0)


def test_cpp_adapter_compiles_against_reference_shaped_types(tmp_path):
    """include/CLUEAlgoGB300.h must compile with PointsCloud/PointsCloudSerial
    shaped like the reference's (src/serial/DataFormats/PointsCloud.h)."""
    src = tmp_path / "adapter.cc"
    src.write_text(
        '#include <vector>\n'
        'struct PointsCloud { std::vector<float> x, y; std::vector<int> layer; std::vector<float> weight; };\n'
        'struct PointsCloudSerial { std::vector<float> x, y; std::vector<int> layer; std::vector<float> weight;\n'
        '  std::vector<float> rho, delta; std::vector<int> nearestHigher; std::vector<std::vector<int>> followers;\n'
        '  std::vector<int> isSeed, clusterIndex; };\n'
        '#include "CLUEAlgoGB300.h"\n'
        'void f(PointsCloud const& pc, PointsCloudSerial& out) {\n'
        '  CLUEAlgoGB300 algo(1.3f, 2.f, 2.f);\n'
        '  algo.makeClusters(pc, out, 1.3f, 2.f, 2.f);\n'
        '}\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
