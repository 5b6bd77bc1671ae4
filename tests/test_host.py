"""Host-side checks that need no GPU: the C-ABI library builds and exports
every symbol of include/gp_ptp.h, the host CHE builder matches the reference,
and the GPU entry points fail loudly (no CPU fallback) when no GPU is there."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import golden_cases, ROOT

CASES = golden_cases()


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "gp_ptp.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gp_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_header_symbol(built_lib):
    syms = header_symbols()
    assert len(syms) >= 14
    L = ctypes.CDLL(built_lib)
    for s in syms:
        assert hasattr(L, s), s
    from gproshan_gb300 import _capi
    assert set(_capi.SIGNATURES) == set(syms)


@pytest.mark.parametrize("name,g", CASES, ids=[c[0] for c in CASES])
def test_che_build_matches_reference(built_lib, name, g):
    from gproshan_gb300 import _capi
    OT, EVT, manifold = _capi.che_build(len(g["xyz"]), g["tri"])
    assert np.array_equal(OT, g["OT"])
    assert np.array_equal(EVT, g["EVT"])
    assert manifold == (not (g["EVT"] == 0xFFFFFFFF).any() or name != "nonmanifold")


def test_che_build_rejects_bad_index(built_lib):
    from gproshan_gb300 import _capi
    with pytest.raises(_capi.GPError):
        _capi.che_build(3, np.array([[0, 1, 5]], np.uint32))


def test_che_class_star_and_link(built_lib):
    from gproshan_gb300 import che, meshgen
    xyz, tri = meshgen.height_field(6, 0)
    m = che(xyz, tri)
    assert m.n_vertices() == 36 and m.n_faces() == 50
    # interior vertex of a grid triangulated with one diagonal per cell has 6 neighbours
    v = 2 * 6 + 2
    assert len(m.star(v)) == 6 and len(m.link(v)) == 6
    # corner: open fan, link has one more entry than the star
    assert len(m.link(0)) == len(m.star(0)) + 1


def test_meshgen_sizes():
    from gproshan_gb300 import meshgen
    xyz, tri = meshgen.icosphere(4, 0.1, 0)
    assert len(xyz) == 10 * 4 ** 4 + 2 and len(tri) == 20 * 4 ** 4
    assert np.allclose(np.linalg.norm(xyz, axis=1), 1.0)
    xyz, tri = meshgen.height_field(64, 0)
    assert len(xyz) == 64 * 64 and len(tri) == 2 * 63 * 63
    xyz, tri = meshgen.torus(40, 25)
    assert len(xyz) == 1000 and len(tri) == 2000


def test_no_gpu_fails_loudly(built_lib):
    """Without a usable GB300 the product path raises; it never computes on the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from gproshan_gb300 import _capi, che, geodesics, meshgen
    with pytest.raises(_capi.GPError) as e:
        _capi.Context(0)
    assert e.value.status == 6  # GP_ERR_NO_DEVICE
    xyz, tri = meshgen.icosphere(2, 0.0, 0)
    with pytest.raises(_capi.GPError):
        geodesics(che(xyz, tri), [0], geodesics.PTP_GPU)


def test_unsupported_options_raise(built_lib):
    from gproshan_gb300 import che, geodesics, meshgen
    xyz, tri = meshgen.icosphere(1, 0.0, 0)
    with pytest.raises(NotImplementedError):
        geodesics(che(xyz, tri), [0], geodesics.FM)


def test_cpp_dropin_shim_compiles_against_reference_headers():
    """The C++ shim that replaces src/cuda/geodesics_ptp*.cu compiles against
    the reference's own headers (FP64 and SINGLE_P builds)."""
    import shutil
    import subprocess
    import oracle
    src = oracle.reference_sources()
    if src is None or not shutil.which("g++"):
        pytest.skip("reference sources (GPROSHAN_REF or the staged copy) or g++ not present")
    ref = os.path.join(src, "include")
    shim = os.path.join(ROOT, "gproshan_gb300", "shim", "geodesics_ptp_gb300.cpp")
    driver = os.path.join(ROOT, "tests", "dropin", "dropin_main.cpp")
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")),
                            "include")
    for src in (shim, driver):
        for extra in ([], ["-DSINGLE_P"]):
            r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-fopenmp", *extra,
                                "-I", os.path.join(ROOT, "oracle", "stubs"), "-I", ref, "-I", cuda_inc,
                                "-I", os.path.join(ROOT, "include"), src], capture_output=True, text=True)
            assert r.returncode == 0, r.stderr


def test_ctypes_struct_layouts_match_the_header(tmp_path):
    """Every struct the ctypes binding mirrors has the header's size and field
    offsets (a C probe compiled against include/gp_ptp.h prints them)."""
    import shutil
    import subprocess
    from gproshan_gb300 import _capi
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    structs = [_capi.gp_ptp_opts, _capi.gp_ptp_stats, _capi.gp_call_stats, _capi.gp_field]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gp_ptp.h"', 'int main(void) {']
    for st in structs:
        name = st.__name__
        lines.append(f'printf("{name} size %zu\\n", sizeof({name}));')
        for fname, _ in st._fields_:
            lines.append(f'printf("{name} {fname} %zu\\n", offsetof({name}, {fname}));')
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            *key, val = line.split()
            got[tuple(key)] = int(val)
    for st in structs:
        name = st.__name__
        assert got[(name, "size")] == ctypes.sizeof(st), name
        for fname, _ in st._fields_:
            assert got[(name, fname)] == getattr(st, fname).offset, (name, fname)
