"""Generate the golden vectors under tests/golden/ from the REFERENCE'S OWN code.

The reference ships no golden vectors or known-answer tests for PTP (its only
harness reads external .off/.exact files that are not distributed), so the
fixtures here are produced by running its unmodified CPU code, compiled by
``make -C oracle ref`` from the reference checkout into oracle/_ref/:

* che(vertices, faces) tables VT / OT / EVT        (src/che.cpp:1254-1362)
* che::compute_toplesets -> rings, sorted, limits  (src/che.cpp:546-593)
* parallel_toplesets_propagation_cpu, FP64 and FP32 builds
                                                   (src/geodesics_ptp.cpp:122-199)

Run from the repository root:
    make -C oracle ref REF=<gproshan checkout>
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from gproshan_gb300 import meshgen  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def grid_with_hole(n=20, seed=0):
    xyz, tri = meshgen.height_field(n, seed)
    # drop the faces of a 4x4 block of cells in the middle: an inner border
    keep = np.ones(len(tri), bool)
    for r in range(n // 2 - 2, n // 2 + 2):
        for c in range(n // 2 - 2, n // 2 + 2):
            cell = r * (n - 1) + c
            keep[2 * cell] = keep[2 * cell + 1] = False
    return xyz, tri[keep]


def bowtie_and_fin():
    """Non-manifold cases: two fans sharing one vertex (a pinch) and an edge
    with three faces (a fin), plus a regular strip around them."""
    xyz, tri = meshgen.height_field(8, 3)
    tri = [list(t) for t in tri]
    nv = len(xyz)
    extra = np.array([[0.5, 0.5, 0.3], [0.6, 0.45, 0.35], [0.4, 0.55, 0.32]])
    xyz = np.concatenate([xyz, extra])
    pinch = 27  # an interior grid vertex
    tri.append([pinch, nv, nv + 1])          # second fan through the pinch vertex
    tri.append([nv + 1, nv, nv + 2])
    tri.append([9, 10, nv + 2])              # fin on grid edge (9, 10)
    return xyz, np.array(tri, dtype=np.uint32)


def two_components():
    a_xyz, a_tri = meshgen.icosphere(2, 0.1, 4)
    b_xyz, b_tri = meshgen.icosphere(2, 0.1, 5)
    b_xyz = b_xyz + np.array([3.0, 0.0, 0.0])
    return np.concatenate([a_xyz, b_xyz]), np.concatenate([a_tri, b_tri + len(a_xyz)]).astype(np.uint32)


CASES = {
    "ico3": (lambda: meshgen.icosphere(3, 0.1, 1), [[0], [5, 17], [3, 3, 9]]),
    "grid24": (lambda: meshgen.height_field(24, 2), [[0], [100, 300], [575]]),
    "grid_hole": (grid_with_hole, [[0], [168], [210]]),
    "nonmanifold": (bowtie_and_fin, [[0], [27], [64, 65]]),
    "two_components": (two_components, [[0], [170]]),
    "torus": (lambda: meshgen.torus(30, 12, seed=3), [[0], [7, 200]]),
}


def main():
    r64 = oracle.RefLib("f64")
    r32 = oracle.RefLib("f32")
    for name, (gen, sources) in CASES.items():
        xyz, tri = gen()
        xyz = np.asarray(xyz, np.float64)
        tri = np.asarray(tri, np.uint32)
        m64 = oracle.RefMesh(r64, xyz, tri)
        m32 = oracle.RefMesh(r32, xyz, tri)
        VT, OT, EVT = m64.tables()
        rec = {"xyz": xyz, "tri": tri, "VT": VT, "OT": OT, "EVT": EVT, "n_sets": np.array(len(sources))}
        for k, src in enumerate(sources):
            rings, srt, lim = m64.toplesets(src)
            if len(lim) < 3 or len(set(src)) != len(src):
                # Undefined behaviour in the reference, so only the toplesets
                # are recorded for these sets: with an isolated source its PTP
                # loop reads limits[2] past the end; with a repeated source
                # `sorted` outgrows n_vertices and the error array indexed by
                # sorted position (src/geodesics_ptp.cpp:225-230, sized
                # n_vertices) is written past its end.
                d64 = np.full(len(xyz), np.nan)
                d32 = np.full(len(xyz), np.nan, np.float32)
            else:
                d64 = m64.ptp_cpu(src, lim, srt, coalescence=False)
                d32 = m32.ptp_cpu(src, lim, srt, coalescence=False)
            rec[f"src{k}"] = np.array(src, np.uint32)
            rec[f"rings{k}"] = rings
            rec[f"sorted{k}"] = srt
            rec[f"limits{k}"] = lim
            rec[f"dist_cpu_f64_{k}"] = d64
            rec[f"dist_cpu_f32_{k}"] = d32
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **rec)
        print(name, len(xyz), "vertices", len(tri), "faces", len(sources), "source sets")


if __name__ == "__main__":
    main()
