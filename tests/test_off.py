"""OFF input: the reader against hand-written files and against the
reference's own che_off (when oracle/_ref is built), and on the GPU the
half-edge tables built in parallel against the host build (exact, including
the non-manifold golden meshes), and a mesh loaded from a file solving like
the same mesh given as arrays."""
import os

import numpy as np
import pytest

from conftest import golden_cases


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


TRI = """OFF
# a square as two triangles
4 2 0
0 0 0
1 0 0
1 1 0
0 1 0.5
3 0 1 2
3 0 2 3
"""

QUAD = """OFF
4 1 0
0 0 0  1 0 0
1 1 0
0 1 0
4 0 1 2 3
"""

COFF = """COFF
3 1 0
0 0 0 255 0 0 255
1 0 0 0 255 0 255
0 1 0 0 0 255 255
3 0 1 2
"""

NOFF = """NOFF
3 1 0
0 0 0 0 0 1
1 0 0 0 0 1
0 1 0 0 0 1
3 2 1 0
"""


def test_off_reader_formats(built_lib, tmp_path):
    from gproshan_gb300 import _capi
    xyz, tri = _capi.off_read(_write(tmp_path, "t.off", TRI))
    assert xyz.shape == (4, 3) and xyz[3, 2] == 0.5
    assert tri.tolist() == [[0, 1, 2], [0, 2, 3]]
    xyz, tri = _capi.off_read(_write(tmp_path, "q.off", QUAD))
    assert tri.tolist() == [[0, 1, 2], [3, 0, 2]]  # the reference's quad split
    xyz, tri = _capi.off_read(_write(tmp_path, "c.off", COFF))
    assert xyz.tolist() == [[0, 0, 0], [1, 0, 0], [0, 1, 0]] and tri.tolist() == [[0, 1, 2]]
    xyz, tri = _capi.off_read(_write(tmp_path, "n.off", NOFF))
    assert tri.tolist() == [[2, 1, 0]] and xyz[1, 0] == 1


@pytest.mark.parametrize("text", [
    "PLY\n3 1 0\n0 0 0\n1 0 0\n0 1 0\n3 0 1 2\n",          # not OFF
    "OFF\n3 1 0\n0 0 0\n1 0 0\n0 1 0\n3 0 1 7\n",          # index out of range
    "OFF\n5 1 0\n0 0 0\n1 0 0\n1 1 0\n0 1 0\n0 2 0\n5 0 1 2 3 4\n",  # pentagon
    "OFF\n3 1 0\n0 0 0\n1 0\n",                             # truncated
])
def test_off_reader_rejects_bad_files(built_lib, tmp_path, text):
    from gproshan_gb300 import _capi
    with pytest.raises(_capi.GPError):
        _capi.off_read(_write(tmp_path, "bad.off", text))


def _ref_lib():
    import oracle
    try:
        return oracle.RefLib("f64")
    except FileNotFoundError:
        pytest.skip("reference build (oracle/_ref) not present")


def _to_off(path, xyz, tri, quads=False):
    with open(path, "w") as f:
        if quads:
            q = tri.reshape(-1, 6)
            # (a,b,c),(d,a,c) pairs written back as quads a b c d
            f.write(f"OFF\n{len(xyz)} {len(q)} 0\n")
            for p in xyz:
                f.write(f"{float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n")
            for r in q:
                f.write(f"4 {r[0]} {r[1]} {r[2]} {r[3]}\n")
        else:
            f.write(f"OFF\n{len(xyz)} {len(tri)} 0\n")
            for p in xyz:
                f.write(f"{float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n")
            for t in tri:
                f.write(f"3 {t[0]} {t[1]} {t[2]}\n")


@pytest.mark.parametrize("quads", [False, True])
def test_off_reader_matches_reference_che_off(built_lib, tmp_path, quads):
    from gproshan_gb300 import _capi, meshgen
    ref = _ref_lib()
    xyz, tri = meshgen.height_field(20, 3)
    if quads:
        tri = tri.reshape(-1, 3)
        # make quad pairs (a,b,c),(d,a,c) from the grid cells
        n = 20
        r, c = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="ij")
        a = (r * n + c).ravel()
        b, d, e = a + 1, a + n, a + n + 1
        tri = np.stack([a, b, e, d, a, e], 1).reshape(-1, 3).astype(np.uint32)
    p = str(tmp_path / "m.off")
    _to_off(p, xyz, tri, quads)
    x1, t1 = _capi.off_read(p)
    x0, VT0, OT0, EVT0 = ref.read_off(p)
    assert np.array_equal(x1, x0)
    assert np.array_equal(t1.reshape(-1), VT0)
    OT1, EVT1, _ = _capi.che_build(len(x1), t1)
    assert np.array_equal(OT1, OT0) and np.array_equal(EVT1, EVT0)


# ---- GPU ----------------------------------------------------------------------

CASES = golden_cases()


@pytest.mark.gpu
@pytest.mark.parametrize("name,g", CASES, ids=[c[0] for c in CASES])
def test_gpu_che_build_equals_host(gpu_ctx, name, g):
    from gproshan_gb300 import _capi
    nv = len(g["xyz"])
    OT0, EVT0, man0 = _capi.che_build(nv, g["tri"])
    OT1, EVT1, man1 = _capi.che_build_device(gpu_ctx, nv, g["tri"])
    assert np.array_equal(OT1, OT0) and np.array_equal(EVT1, EVT0) and man1 == man0


@pytest.mark.gpu
def test_gpu_che_build_random_soups(gpu_ctx):
    """Triangle soups over few vertices: edges shared by many triangles in
    both directions, repeated triangles, degenerate triangles."""
    from gproshan_gb300 import _capi
    rng = np.random.default_rng(3)
    for trial in range(20):
        nv = int(rng.integers(3, 12))
        tri = rng.integers(0, nv, size=(int(rng.integers(1, 10)), 3)).astype(np.uint32)
        OT0, EVT0, man0 = _capi.che_build(nv, tri)
        OT1, EVT1, man1 = _capi.che_build_device(gpu_ctx, nv, tri)
        assert np.array_equal(OT1, OT0), trial
        assert np.array_equal(EVT1, EVT0) and man1 == man0, trial


@pytest.mark.gpu
def test_gpu_mesh_from_off_solves_like_arrays(gpu_ctx, tmp_path):
    from gproshan_gb300 import _capi, meshgen
    xyz, tri = meshgen.icosphere(4, 0.1, 5)
    p = str(tmp_path / "ico.off")
    _to_off(p, xyz, tri)
    m_file = _capi.mesh_from_off(gpu_ctx, p)
    m_arr = _capi.DeviceMesh(gpu_ctx, xyz, tri)
    assert m_file.n_vertices == len(xyz) and m_file.n_faces == len(tri)
    a, _, sa = _capi.ptp(m_file, [0, 100])
    b, _, sb = _capi.ptp(m_arr, [0, 100])
    assert np.array_equal(a, b) and sa.n_iter == sb.n_iter
