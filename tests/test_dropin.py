"""The C++ drop-in, linked and run: gproshan_gb300/shim/geodesics_ptp_gb300.cpp
compiled together with the reference's own che / vertex / geodesics_ptp sources
(the che class the reference's callers hold) and libgp_ptp.so, driven by
tests/dropin/dropin_main.cpp through the reference's public entry points
(include/geodesics_ptp.h:34-42).  Needs the reference's sources (GPROSHAN_REF
or the staged copy) and g++; skipped without them.

Checks, default build (distance_t = double, so the FP64 path):
* parallel_toplesets_propagation_gpu: distances bit-exact with the oracle,
  labels with the oracle's GPU label rule;
* parallel_toplesets_propagation_coalescence_gpu: the same on reached
  vertices, the caller's distance and label kept on unreached ones
  (src/cuda/geodesics_ptp_coalescence.cu:62-86);
* a cudaDeviceReset between calls (gproshan's heat-flow code issues one) does
  not break the next call;
* farthest_point_sampling_ptp_gpu: the oracle's samples and radius.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dropin_exe(tmp_path_factory, built_lib):
    import oracle
    ref = oracle.reference_sources()
    if ref is None or not shutil.which("g++"):
        pytest.skip("reference sources (GPROSHAN_REF or the staged copy) or g++ not present")
    cuda = os.path.dirname(os.path.dirname(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"))
    out = str(tmp_path_factory.mktemp("dropin") / "dropin")
    lib_dir = os.path.dirname(built_lib)
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-DNDEBUG", "-w",
           "-I", os.path.join(ROOT, "oracle", "stubs"), "-I", os.path.join(ref, "include"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "dropin", "dropin_main.cpp"),
           os.path.join(ROOT, "gproshan_gb300", "shim", "geodesics_ptp_gb300.cpp"),
           *[os.path.join(ref, "src", f) for f in ("che.cpp", "vertex.cpp", "che_off.cpp", "geodesics_ptp.cpp")],
           "-L", lib_dir, "-lgp_ptp", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


def _run(exe, d, xyz, tri, src, n_fps, env=None):
    os.makedirs(d, exist_ok=True)
    np.ascontiguousarray(xyz, np.float64).tofile(os.path.join(d, "xyz.f64"))
    np.ascontiguousarray(tri, np.uint32).tofile(os.path.join(d, "tri.u32"))
    np.asarray(src, np.uint32).tofile(os.path.join(d, "src.u32"))
    np.asarray([n_fps], np.uint32).tofile(os.path.join(d, "fps.u32"))
    r = subprocess.run([exe, d], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    rd = lambda n, t: np.fromfile(os.path.join(d, n), dtype=t)
    return {k: rd(k, np.float64) for k in ("gpu.dist", "gpu_reset.dist", "coal.dist")} | \
           {k: rd(k, np.uint32) for k in ("gpu.cl", "coal.cl", "fps_samples.u32")} | {"fps.max": rd("fps.max", np.float64)}


def test_dropin_entry_points_match_the_oracle(dropin_exe, oracle_lib, tmp_path):
    from gproshan_gb300 import meshgen
    xyz, tri = meshgen.icosphere(4, 0.1, 3)
    src = [0, 1500, 2000]
    out = _run(dropin_exe, str(tmp_path / "ico"), xyz, tri, src, 9)
    om = oracle_lib.Mesh(xyz, tri)
    ref = oracle_lib.ptp(om, src, clusters=True)
    assert np.array_equal(out["gpu.dist"], ref["dist"])
    assert np.array_equal(out["gpu.cl"], ref["clusters"])
    assert np.array_equal(out["coal.dist"], ref["dist"])       # every vertex reached
    assert np.array_equal(out["coal.cl"], ref["clusters"])
    assert np.array_equal(out["gpu_reset.dist"], out["gpu.dist"])
    s_ref, md_ref = oracle_lib.fps(om, 9, [0])
    assert np.array_equal(out["fps_samples.u32"], s_ref)
    assert out["fps.max"][0] == md_ref


def test_dropin_coalescence_keeps_caller_values_on_unreached_vertices(dropin_exe, oracle_lib, tmp_path):
    """Two components, sources in the first: the multi-source entry writes INF
    on the second, the coalescence entry leaves the caller's -7 and 12345."""
    from gproshan_gb300 import meshgen
    x1, t1 = meshgen.icosphere(3, 0.1, 1)
    x2, t2 = meshgen.height_field(20, 2)
    xyz = np.concatenate([x1, x2 + np.array([3.0, 0.0, 0.0])])
    tri = np.concatenate([t1, t2 + len(x1)]).astype(np.uint32)
    src = [5, 300]
    out = _run(dropin_exe, str(tmp_path / "two"), xyz, tri, src, 1)
    om = oracle_lib.Mesh(xyz, tri)
    ref = oracle_lib.ptp(om, src, clusters=True)
    first = np.arange(len(xyz)) < len(x1)
    assert np.array_equal(out["gpu.dist"], ref["dist"]) and np.isinf(out["gpu.dist"][~first]).all()
    assert np.array_equal(out["coal.dist"][first], ref["dist"][first])
    assert (out["coal.dist"][~first] == -7).all() and (out["coal.cl"][~first] == 12345).all()
    assert np.array_equal(out["coal.cl"][first], ref["clusters"][first])
    assert np.array_equal(out["gpu_reset.dist"], out["gpu.dist"])


def test_dropin_fp32_opt_in(dropin_exe, oracle_lib, tmp_path):
    """GP_PTP_PRECISION=f32: a double build computes in FP32 and still writes
    doubles: within 1e-5 of the FP64 oracle on the float-rounded coordinates
    the FP32 path reads, labels and FPS samples equal to the oracle's."""
    from gproshan_gb300 import meshgen
    xyz, tri = meshgen.icosphere(4, 0.1, 3)
    src = [0, 1500, 2000]
    env = dict(os.environ, GP_PTP_PRECISION="f32")
    out = _run(dropin_exe, str(tmp_path / "f32"), xyz, tri, src, 9, env=env)
    om = oracle_lib.Mesh(xyz, tri)
    x32 = xyz.astype(np.float32).astype(np.float64)
    ref = oracle_lib.ptp(om, src, clusters=True, xyz=x32)
    assert oracle_lib.max_rel_err(out["gpu.dist"], ref["dist"]) <= 1e-5
    assert not np.array_equal(out["gpu.dist"], oracle_lib.ptp(om, src)["dist"])  # not the FP64 path
    assert np.array_equal(out["gpu.cl"], ref["clusters"])
    assert np.array_equal(out["fps_samples.u32"], oracle_lib.fps(om, 9, [0])[0])
