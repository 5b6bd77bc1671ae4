"""The CPU oracle (oracle/ptp_oracle.c) pinned against the golden vectors made
by the reference's own compiled code (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from conftest import golden_cases, ROOT

CASES = golden_cases()


@pytest.mark.parametrize("name,g", CASES, ids=[c[0] for c in CASES])
def test_che_tables_match_reference(oracle_lib, name, g):
    m = oracle_lib.Mesh(g["xyz"], g["tri"])
    assert np.array_equal(m.VT, g["VT"])
    assert np.array_equal(m.OT, g["OT"])
    assert np.array_equal(m.EVT, g["EVT"])


@pytest.mark.parametrize("name,g", CASES, ids=[c[0] for c in CASES])
def test_toplesets_match_reference(oracle_lib, name, g):
    m = oracle_lib.Mesh(g["xyz"], g["tri"])
    for k in range(int(g["n_sets"])):
        rings, srt, lim = oracle_lib.toplesets(m, g[f"src{k}"])
        assert np.array_equal(rings, g[f"rings{k}"]), (name, k)
        assert np.array_equal(srt, g[f"sorted{k}"]), (name, k)
        assert np.array_equal(lim, g[f"limits{k}"]), (name, k)


@pytest.mark.parametrize("name,g", CASES, ids=[c[0] for c in CASES])
def test_ptp_cpu_buffer_bit_exact(oracle_lib, name, g):
    """The oracle's CPU-returned buffer equals the reference CPU PTP bit for bit."""
    m = oracle_lib.Mesh(g["xyz"], g["tri"])
    checked = 0
    for k in range(int(g["n_sets"])):
        ref = g[f"dist_cpu_f64_{k}"]
        if np.isnan(ref).all():
            continue  # undefined behaviour in the reference for this set
        out = oracle_lib.ptp(m, g[f"src{k}"], g[f"limits{k}"], g[f"sorted{k}"])
        assert np.array_equal(out["dist_cpu"], ref), (name, k)
        checked += 1
    assert checked >= 1


def test_golden_has_nonmanifold_and_borders():
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "nonmanifold.npz")))
    assert (g["EVT"] == 0xFFFFFFFF).any()  # a vertex dropped as non-manifold
    h = dict(np.load(os.path.join(ROOT, "tests", "golden", "grid_hole.npz")))
    assert (h["OT"] == 0xFFFFFFFF).sum() > 0  # border half-edges


def test_isolated_source_runs_no_sweep(oracle_lib):
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "grid_hole.npz")))
    m = oracle_lib.Mesh(g["xyz"], g["tri"])
    src = g["src2"]
    assert len(g["limits2"]) == 2
    out = oracle_lib.ptp(m, src, g["limits2"], g["sorted2"])
    assert out["n_iter"] == 0
    d = out["dist"]
    assert d[src[0]] == 0 and np.isinf(np.delete(d, src[0])).all()


def test_gpu_and_cpu_entry_points_differ_by_one_sweep(oracle_lib):
    """The reference CPU entry points return the buffer one sweep older than
    the GPU ones; the oracle exposes both."""
    from gproshan_gb300 import meshgen
    xyz, tri = meshgen.height_field(32, 1)
    m = oracle_lib.Mesh(xyz, tri)
    out = oracle_lib.ptp(m, [0])
    assert out["n_iter"] > 0
    assert not np.array_equal(out["dist"], out["dist_cpu"])


def test_replay_reproduces_schedule(oracle_lib):
    from gproshan_gb300 import meshgen
    xyz, tri = meshgen.icosphere(3, 0.1, 7)
    m = oracle_lib.Mesh(xyz, tri)
    _, srt, lim = oracle_lib.toplesets(m, [4])
    out = oracle_lib.ptp(m, [4], lim, srt, trace=True)
    rep = oracle_lib.ptp_replay(m, [4], lim, srt, out["trace"])
    assert np.array_equal(rep, out["dist"])


@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libref_f64.so")),
                    reason="reference build (oracle/_ref) not present")
def test_oracle_vs_reference_random_meshes(oracle_lib):
    """Fresh seeded meshes, both the oracle and the reference's own code."""
    from gproshan_gb300 import meshgen
    R = oracle_lib.RefLib("f64")
    rng = np.random.default_rng(11)
    for seed in range(3):
        xyz, tri = meshgen.height_field(int(rng.integers(12, 40)), seed)
        m = oracle_lib.Mesh(xyz, tri)
        rm = oracle_lib.RefMesh(R, xyz, tri)
        src = list(rng.choice(m.nv, size=int(rng.integers(1, 4)), replace=False))
        r1, s1, l1 = oracle_lib.toplesets(m, src)
        r2, s2, l2 = rm.toplesets(src)
        assert np.array_equal(r1, r2) and np.array_equal(s1, s2) and np.array_equal(l1, l2)
        out = oracle_lib.ptp(m, src, l1, s1)
        assert np.array_equal(out["dist_cpu"], rm.ptp_cpu(src, l2, s2))


def _closed_form_cases():
    """A flat grid (exact geodesic = Euclidean distance) and a unit icosphere
    (exact = great-circle angle), with their sources."""
    from gproshan_gb300 import meshgen
    flat, ft = meshgen.height_field(101, 0)
    flat = flat.copy()
    flat[:, 2] = 0.0
    fs = 50 * 101 + 50
    sph, st = meshgen.icosphere(5, 0.0, 0)
    sph = sph / np.linalg.norm(sph, axis=1)[:, None]
    return [("flat101", flat, ft, fs, np.linalg.norm(flat - flat[fs], axis=1)),
            ("sphere_L5", sph, st, 0, np.arccos(np.clip(sph @ sph[0], -1.0, 1.0)))]


def mean_rel_err_pct(dist, exact):
    """compute_error of the reference's harness (src/test_geodesics_ptp.cpp:362-371):
    mean relative error in %, over the vertices whose exact distance is > 0."""
    m = exact > 0
    return 100.0 * float(np.mean(np.abs(dist[m] - exact[m]) / exact[m]))


@pytest.mark.parametrize("case", [0, 1], ids=["flat101", "sphere_L5"])
def test_accuracy_against_closed_form_geodesics(oracle_lib, case):
    """The PTP algorithm's own accuracy, the quantity the reference's
    test_geodesics harness reports against exact distances: ~1.4 % mean
    relative error on a flat grid, ~1.0 % on a unit sphere."""
    name, xyz, tri, src, exact = _closed_form_cases()[case]
    m = oracle_lib.Mesh(xyz, tri)
    r = oracle_lib.ptp(m, [src])
    err = mean_rel_err_pct(r["dist"], exact)
    assert err < {"flat101": 1.5, "sphere_L5": 1.0}[name], (name, err)
