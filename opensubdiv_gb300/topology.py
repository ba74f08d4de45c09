"""Uniform-refinement stencil tables for synthetic cages (libosd_gb300_topology.so).

This is the workload generator: it produces Far::StencilTable-shaped tables (sizes,
offsets, control indices, weights; factorized to the control vertices) for closed
Catmull-Clark and Loop cages with semi-sharp creases, and bilinear limit stencils with du/dv
weights on a uniformly refined Catmull-Clark cage.  See csrc/host/uniform_refine.cpp for the
rules it restates.  Tables are validated against the reference's own Far tables in
tests/test_topology.py.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_path = None


def use_library(path: str) -> None:
    """Loads the generator from `path` instead of the package's own build (a process that
    must not map this package's libraries -- the CPU reference timing -- builds the same
    sources elsewhere).  Must be called before the first load()."""
    global _path
    if _lib is not None:
        raise RuntimeError("the generator library is already loaded")
    _path = path


def load():
    global _lib
    if _lib is None:
        path = _path or _build.TOPO_LIB
        if _path is None and not os.path.exists(path):
            _build.build_topology()
        lib = C.CDLL(path)
        vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
        lib.GB300TopologyCreate.restype = vp
        lib.GB300TopologyCreate.argtypes = [i32, i32, i32, vp, vp, i32, vp, vp]
        lib.GB300TopologyDestroy.argtypes = [vp]
        lib.GB300TopologyRefineUniform.argtypes = [vp, i32]
        lib.GB300TopologyGetNumVertices.argtypes = [vp, i32]
        lib.GB300TopologyGetNumPtexFaces.argtypes = [vp]
        lib.GB300TopologyStencilCounts.argtypes = [vp, i32, i32, C.POINTER(i32), C.POINTER(i64)]
        lib.GB300TopologyStencilCopy.argtypes = [vp, i32, i32, vp, vp, vp, vp]
        lib.GB300TopologyLimitStencils.argtypes = [vp, i32, vp, vp, vp]
        lib.GB300TopologyLimitStencilNnz.restype = i64
        lib.GB300TopologyLimitStencilNnz.argtypes = [vp]
        lib.GB300TopologyLimitStencilCopy.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        lib.GB300TopologyGetLastError.restype = C.c_char_p
        lib.GB300TopologySetNumThreads.argtypes = [i32]
        lib.GB300TopologySetNumThreads.restype = None
        lib.GB300TopologyRefineTopology.argtypes = [vp, i32]
        lib.GB300TopologyMaskCounts.argtypes = [vp, i32, vp, vp]
        lib.GB300TopologyMaskCopy.argtypes = [vp, vp, vp, vp]
        _lib = lib
    return _lib


def _err():
    return load().GB300TopologyGetLastError().decode()


class UniformRefiner:
    """Uniform refinement of a shapes.Cage (Catmull-Clark or Loop, closed, with creases)."""

    def __init__(self, cage, level: int, stencils: bool = True):
        """stencils=False refines the topology only (for masks() / the GPU factory)."""
        lib = load()
        self.cage = cage
        self.level = level
        cv = np.ascontiguousarray(cage.crease_verts, np.int32).reshape(-1)
        cs = np.ascontiguousarray(cage.crease_sharpness, np.float32)
        self._keep = (cv, cs)
        self.h = lib.GB300TopologyCreate(cage.scheme, cage.num_vertices, cage.num_faces,
                                         cage.verts_per_face.ctypes.data,
                                         cage.face_verts.ctypes.data, len(cs),
                                         cv.ctypes.data if len(cv) else None,
                                         cs.ctypes.data if len(cs) else None)
        if not self.h:
            raise ValueError(_err())
        refine = lib.GB300TopologyRefineUniform if stencils else lib.GB300TopologyRefineTopology
        if refine(self.h, level) != 0:
            raise ValueError(_err())

    def __del__(self):
        if getattr(self, "h", None):
            load().GB300TopologyDestroy(self.h)
            self.h = None

    def num_vertices(self, level):
        return load().GB300TopologyGetNumVertices(self.h, level)

    def num_ptex_faces(self):
        return load().GB300TopologyGetNumPtexFaces(self.h)

    def stencil_table(self, first: int | None = None, last: int | None = None):
        """Factorized stencils of levels [first, last] (default: the finest level only, i.e.
        StencilTableFactory with generateIntermediateLevels=false)."""
        lib = load()
        last = self.level if last is None else last
        first = last if first is None else first
        n, nnz = C.c_int(0), C.c_int64(0)
        if lib.GB300TopologyStencilCounts(self.h, first, last, C.byref(n), C.byref(nnz)):
            raise ValueError(_err())
        sizes = np.empty(n.value, np.int32)
        offsets = np.empty(n.value, np.int32)
        idx = np.empty(nnz.value, np.int32)
        w = np.empty(nnz.value, np.float32)
        lib.GB300TopologyStencilCopy(self.h, first, last, sizes.ctypes.data, offsets.ctypes.data,
                                     idx.ctypes.data, w.ctypes.data)
        return dict(sizes=sizes, offsets=offsets, indices=idx, weights=w)

    def masks(self, level):
        """Subdivision masks of the level-`level` vertices in Far::PrimvarRefiner's form
        (per child: (global source, float32 weight) in call order; Catmark edge and vertex
        points name the level's own face points): dict of int64 offsets, int32 sources,
        float32 weights -- the input of GB300StencilTableFactory."""
        lib = load()
        n, nnz = C.c_int(0), C.c_int64(0)
        if lib.GB300TopologyMaskCounts(self.h, level, C.byref(n), C.byref(nnz)):
            raise ValueError(_err())
        off = np.empty(n.value + 1, np.int64)
        idx = np.empty(nnz.value, np.int32)
        w = np.empty(nnz.value, np.float32)
        lib.GB300TopologyMaskCopy(self.h, off.ctypes.data, idx.ctypes.data, w.ctypes.data)
        return dict(offsets=off, sources=idx, weights=w)

    def factory_masks(self):
        """(number of control vertices, masks of levels 1..level)."""
        return self.cage.num_vertices, [self.masks(l) for l in range(1, self.level + 1)]

    def limit_stencil_table(self, faces, u, v):
        """Bilinear limit stencils with du/dv weights at (ptex face, u, v) locations."""
        lib = load()
        faces = np.ascontiguousarray(faces, np.int32)
        u = np.ascontiguousarray(u, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        m = lib.GB300TopologyLimitStencils(self.h, len(faces), faces.ctypes.data, u.ctypes.data,
                                           v.ctypes.data)
        if m < 0:
            raise ValueError(_err())
        nnz = lib.GB300TopologyLimitStencilNnz(self.h)
        out = dict(sizes=np.empty(m, np.int32), offsets=np.empty(m, np.int32),
                   indices=np.empty(nnz, np.int32), weights=np.empty(nnz, np.float32),
                   du_weights=np.empty(nnz, np.float32), dv_weights=np.empty(nnz, np.float32))
        lib.GB300TopologyLimitStencilCopy(self.h, *[out[k].ctypes.data for k in (
            "sizes", "offsets", "indices", "weights", "du_weights", "dv_weights")])
        return out
