"""Host mirror of gproshan's compact half-edge mesh (``che``, include/che.h:27-130),
reduced to what the PTP geodesics path reads: the geometry table GT, the vertex
table VT, the opposite table OT and the extra vertex table EVT, plus
``compute_toplesets`` (now run on the GPU).

OT/EVT are built by the library's host code (``gp_che_build``) with the
reference's matching and non-manifold rules (che::update_evt_ot_et,
src/che.cpp:1295-1362).
"""
from __future__ import annotations

import numpy as np

from . import _capi

NIL = _capi.NIL


def next_he(he: int) -> int:
    """next(he) (src/che.cpp:24-28)."""
    return NIL if he == NIL else 3 * (he // 3) + (he + 1) % 3


def prev_he(he: int) -> int:
    """prev(he) (src/che.cpp:30-34)."""
    return NIL if he == NIL else 3 * (he // 3) + (he + 2) % 3


class che:
    """Triangle mesh in compact half-edge form."""

    P = 3

    def __init__(self, vertices, faces):
        self.GT = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        self.VT = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1)
        if len(self.VT) % 3:
            raise ValueError("faces must be triangles")
        self.OT, self.EVT, self.manifold = _capi.che_build(len(self.GT), self.VT)
        self._device = {}
        self.filename = ""

    # -- sizes and tables (che.h:81-97) ---------------------------------
    def n_vertices(self) -> int:
        return len(self.GT)

    def n_faces(self) -> int:
        return len(self.VT) // 3

    def n_half_edges(self) -> int:
        return len(self.VT)

    def gt(self, v: int):
        return self.GT[v]

    def vt(self, he: int) -> int:
        return int(self.VT[he])

    def ot(self, he: int) -> int:
        return int(self.OT[he])

    def evt(self, v: int) -> int:
        return int(self.EVT[v])

    def is_manifold(self) -> bool:
        return self.manifold

    # -- star and link (che.cpp:94-112), for inspection ------------------
    def star(self, v: int):
        out = []
        stop = self.evt(v)
        he = stop
        while he != NIL:
            out.append(he)
            he = self.ot(prev_he(he))
            if he == stop:
                he = NIL
        return out

    def link(self, v: int):
        out = []
        for he in self.star(v):
            out.append(next_he(he))
            if self.ot(prev_he(he)) == NIL:
                out.append(prev_he(he))
        return out

    # -- device copy ------------------------------------------------------
    def device(self, ctx: _capi.Context | None = None) -> _capi.DeviceMesh:
        """The gp_mesh of this mesh on ``ctx`` (uploaded once, then reused)."""
        ctx = ctx or _capi.default_context()
        key = id(ctx)
        m = self._device.get(key)
        if m is None:
            m = _capi.DeviceMesh(ctx, self.GT, self.VT, self.OT, self.EVT)
            self._device[key] = m
        return m

    def compute_toplesets(self, sources, k: int = NIL, ctx=None):
        """(toplesets, sorted, limits) as che::compute_toplesets returns them
        (src/che.cpp:546-593), computed on the GPU."""
        if k != NIL:
            raise NotImplementedError("the level limit k is not used by the PTP path")
        return _capi.toplesets(self.device(ctx), sources)


class che_off(che):
    """A mesh read from an OFF file (che_off, include/che_off.h:11-21;
    src/che_off.cpp:28-79): OFF/COFF/NOFF, quads split as the reference
    splits them."""

    def __init__(self, file: str):
        xyz, tri = _capi.off_read(file)
        super().__init__(xyz, tri)
        self.filename = file
