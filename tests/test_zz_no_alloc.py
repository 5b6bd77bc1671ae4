"""gp_toplesets_noalloc: the toplesets entry point that allocates no device memory.

It serves callers that may not allocate device memory while they work (an
application that gave all device memory to its own pool up front, or a
latency-critical loop where cudaMalloc/cudaFree are not allowed): its BFS
scratch is a fixed array inside the library.  This file is collected last so
that a run stopping at the first failure has run every other test first; it
also passes on its own in a fresh process (it makes its own context).

The checks: two calls in a row through the C ABI, each compared bit for bit
with the allocating entry point gp_toplesets (toplesets are integer outputs, so
the tolerance is exact equality); a mesh with valence-64 poles (links longer
than the 8-entry rows, read from the CSR lists) likewise; a source out of range
reports zero limits; and a mesh above the array's 2^20-vertex limit is refused
with GP_ERR_CAPACITY.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GP_ERR_CAPACITY = 8


def _run_noalloc(L, mesh, sources, torch, nl_out=None):
    nv = mesh.n_vertices
    dev = torch.device("cuda")
    src = torch.tensor(np.asarray(sources, np.int64).astype(np.int32), device=dev)
    rings = torch.empty(nv, dtype=torch.int32, device=dev)
    srt = torch.empty(nv + len(sources), dtype=torch.int32, device=dev)
    lim = torch.empty(nv + 2, dtype=torch.int32, device=dev)
    nl = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    st = L.gp_toplesets_noalloc(mesh.handle, src.data_ptr(), len(sources), rings.data_ptr(), srt.data_ptr(),
                                nv + len(sources), lim.data_ptr(), nv + 2, nl.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    n = int(nl.item())
    if nl_out is not None:
        nl_out.append(n)
    as_u32 = lambda t: t.cpu().numpy().view(np.uint32)
    return st, as_u32(rings), as_u32(srt), as_u32(lim)[:n]


def test_noalloc_toplesets_equal_the_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from gproshan_gb300 import _capi, build, meshgen

    build.build()
    torch.cuda.set_device(0)
    ctx = _capi.Context(0)
    L = _capi.lib()
    xyz, tri = meshgen.height_field(120, 7)
    mesh = _capi.DeviceMesh(ctx, xyz, tri)
    # two calls in a row: the second must not see the first's leftovers
    for sources in ([5], [17, 9000, 14399]):
        st, rings, srt, lim = _run_noalloc(L, mesh, sources, torch)
        assert st == 0
        r0, s0, l0 = _capi.toplesets(mesh, sources)
        assert np.array_equal(lim, l0)
        assert np.array_equal(rings, r0)
        assert np.array_equal(srt[:int(l0[-1])], s0)


def test_noalloc_refuses_meshes_above_its_limit():
    torch = pytest.importorskip("torch")
    from gproshan_gb300 import _capi, build, meshgen

    build.build()
    torch.cuda.set_device(0)
    ctx = _capi.Context(0)
    L = _capi.lib()
    xyz, tri = meshgen.height_field(1025, 1)  # 1,050,625 vertices > 2^20
    mesh = _capi.DeviceMesh(ctx, xyz, tri)
    st, _, _, _ = _run_noalloc(L, mesh, [0], torch)
    assert st == GP_ERR_CAPACITY


def test_noalloc_high_valence_rows_and_bad_source():
    torch = pytest.importorskip("torch")
    from gproshan_gb300 import _capi, build
    from test_gpu_parity import _uv_sphere

    build.build()
    torch.cuda.set_device(0)
    ctx = _capi.Context(0)
    L = _capi.lib()
    xyz, tri = _uv_sphere(64, 48)
    mesh = _capi.DeviceMesh(ctx, xyz, tri)
    for sources in ([0], [len(xyz) - 1, 700]):
        st, rings, srt, lim = _run_noalloc(L, mesh, sources, torch)
        assert st == 0
        r0, s0, l0 = _capi.toplesets(mesh, sources)
        assert np.array_equal(lim, l0) and np.array_equal(rings, r0)
        assert np.array_equal(srt[:int(l0[-1])], s0)
    got = []
    st, _, _, _ = _run_noalloc(L, mesh, [3, len(xyz)], torch, got)
    assert st == 0 and got == [0]
    # and the next call is unaffected
    st, rings, _, lim = _run_noalloc(L, mesh, [0], torch)
    r0, _, l0 = _capi.toplesets(mesh, [0])
    assert st == 0 and np.array_equal(lim, l0) and np.array_equal(rings, r0)
