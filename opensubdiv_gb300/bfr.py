"""Bfr tessellation and limit evaluation of a whole mesh on the device.

Mirrors the reference's Bfr classes for the tessellate-and-evaluate loop its tutorials run
face by face (tutorials/bfr/tutorial_1_2/bfr_tutorial_1_2.cpp:170-238):

* :class:`Parameterization` -- Bfr::Parameterization (bfr/parameterization.h:48-190): the
  (u,v) domain of a face, quad, triangle or quad sub-faces of an N-gon;
* :class:`TessellationOptions` -- Bfr::Tessellation::Options (bfr/tessellation.h:60-100);
* :class:`Tessellation` -- Bfr::Tessellation of one face (bfr/tessellation.h:142-262), its
  coords and facets computed on the device;
* :class:`MeshTessellation` -- every face of a mesh at once (GB300TessellationCount /
  GB300TessellationGenerate): coords, facets with mesh-wide indices, and the PatchCoord of
  every coord on a device patch table, which :meth:`MeshTessellation.Evaluate` turns into
  limit positions and derivatives (Bfr::Surface::Evaluate, bfr/surface.h:227-242).

There is no CPU path: the device library must load, or every call raises.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import GB300Error, check, last_error  # noqa: F401
from .evaluator import _ptr, _stream

# Bfr::Limits::MaxFaceSize (bfr/limits.h:43) and the short range of rates (tessellation.cpp:2091)
MAX_FACE_SIZE = 65535
MAX_RATE = 32767


class Parameterization:
    """Bfr::Parameterization of a face of `face_size` vertices for a scheme whose regular face
    has `regular_face_size` vertices (4: Catmark / Bilinear, 3: Loop)."""

    QUAD, TRI, QUAD_SUBFACES = 0, 1, 2

    def __init__(self, regular_face_size: int, face_size: int):
        self.regular_face_size = int(regular_face_size)
        self._type = self.QUAD if regular_face_size == 4 else self.TRI
        self._size = int(face_size)
        self._udim = 0
        if face_size != regular_face_size:
            if face_size < 3 or face_size > MAX_FACE_SIZE or regular_face_size == 3:
                self._size = 0
            else:
                self._type = self.QUAD_SUBFACES
                self._udim = (2 + (face_size > 4)) if face_size < 10 else \
                    1 + int(math.sqrt(np.float32(face_size - 1)))

    def IsValid(self) -> bool: return self._size > 0
    def GetType(self) -> int: return self._type
    def GetFaceSize(self) -> int: return self._size
    def HasSubFaces(self) -> bool: return self._type == self.QUAD_SUBFACES

    def GetVertexCoord(self, vertex: int):
        if self._type == self.QUAD:
            return (float(bool(vertex) and vertex < 3), float(vertex > 1))
        if self._type == self.TRI:
            return (float(vertex == 1), float(vertex == 2))
        return (float(vertex % self._udim), float(vertex // self._udim))

    def GetCenterCoord(self):
        c = np.float32(1.0) / np.float32(3.0) if self._type == self.TRI else np.float32(0.5)
        return (float(c), float(c))


class TessellationOptions(C.Structure):
    """Bfr::Tessellation::Options: facet size 3 or 4, quad preservation, strides (0 =
    defaults: 2 floats between coords, the facet size between facets)."""

    _fields_ = [("facetSize", C.c_int), ("preserveQuads", C.c_int), ("coordStride", C.c_int),
                ("facetStride", C.c_int)]

    def __init__(self, facet_size=3, preserve_quads=False, coord_stride=0, facet_stride=0):
        super().__init__(int(facet_size), int(bool(preserve_quads)), int(coord_stride),
                         int(facet_stride))

    def SetFacetSize(self, n):
        self.facetSize = 4 if n == 4 else 3
        return self

    def PreserveQuads(self, on=True):
        self.preserveQuads = int(bool(on))
        return self

    def GetFacetSize(self) -> int: return 4 if self.facetSize == 4 else 3


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise GB300Error(2, "Bfr tessellation needs a CUDA device")
    return torch


def EdgeRates(face_sizes, face_verts, points, interval, max_rate=10, points_per_corner=False,
              stride=3, stream=None):
    """Per-edge rates from edge lengths, as the reference's Bfr tutorial 2.1 computes them
    (GB300TessellationEdgeRates): rate 1 + int(length / interval) capped at max_rate, lengths
    between the points of consecutive face corners -- mesh-vertex points named by face_verts
    (the tutorial's hull option), or one point per face corner (its limit option).  Returns
    (rate_offsets [faces + 1], rates [corners]) as int32 CUDA tensors, ready for
    MeshTessellation(rates=..., rate_offsets=...)."""
    torch = _torch()
    dev = torch.device("cuda")

    def on_device(x, dtype):
        t = x if hasattr(x, "data_ptr") else torch.from_numpy(np.ascontiguousarray(x))
        return t.to(dev, dtype).contiguous()

    sizes = on_device(face_sizes, torch.int32)
    fv = on_device(face_verts, torch.int32)
    pts = on_device(points, torch.float32).reshape(-1)
    nf, nc = int(sizes.numel()), int(fv.numel())
    offsets = torch.empty(nf + 1, dtype=torch.int32, device=dev)
    rates = torch.empty(max(nc, 1), dtype=torch.int32, device=dev)
    check(_lib.load().GB300TessellationEdgeRates(
        nf, _ptr(sizes), _ptr(fv), nc, _ptr(pts), int(pts.numel()) // stride, int(stride),
        int(bool(points_per_corner)), float(interval), int(max_rate), _ptr(offsets),
        _ptr(rates), _stream(stream)))
    return offsets, rates[:nc]


class SharedPoints:
    """The shared points of MeshTessellation.Share (attributes set there; the full-capacity
    buffers behind patch_coords, coords and faces are kept for reuse through `out`)."""
    num_points = 0
    point_offsets = patch_coords = coords = faces = vertex_points = edge_points = None
    _pc = _coords = _faces = None


class MeshTessellation:
    """Bfr::Tessellation of every face of a mesh, on the device.

    face_sizes: int32 face vertex counts (host array or CUDA tensor).  Rates follow
    GB300TessellationCount: `uniform_rate` for all faces, or `rates` (one per face, or with
    `rate_offsets` a per-face run of Tessellation(p, numRates, rates) rates).  A face with an
    invalid tessellation (rate < 1, a size the scheme rejects) gets nothing -- give holes a
    rate of 0.
    """

    def __init__(self, regular_face_size, face_sizes, uniform_rate=None, rates=None,
                 rate_offsets=None, options=None, stream=None):
        torch = _torch()
        dev = torch.device("cuda")

        def on_device(x):
            if x is None:
                return None
            t = x if hasattr(x, "data_ptr") else torch.from_numpy(np.ascontiguousarray(x, np.int32))
            return t.to(dev, torch.int32).contiguous()

        if rates is None and uniform_rate is None:
            raise ValueError("give uniform_rate or rates")
        self.regular_face_size = int(regular_face_size)
        self.face_sizes = on_device(face_sizes)
        self.rates = on_device(rates)
        self.rate_offsets = on_device(rate_offsets)
        self.uniform_rate = int(uniform_rate) if rates is None else 0
        self.options = options if options is not None else TessellationOptions()
        self.num_faces = int(self.face_sizes.numel())
        self.stream = stream
        n1 = self.num_faces + 1
        self.coord_offsets = torch.zeros(n1, dtype=torch.int64, device=dev)
        self.facet_offsets = torch.zeros(n1, dtype=torch.int64, device=dev)
        self.ptex_offsets = torch.zeros(n1, dtype=torch.int64, device=dev)
        self.Count()

    def Count(self):
        """(Re)computes the per-face offsets and the totals (GB300TessellationCount; reads the
        totals back, so it waits for the stream)."""
        totals = (C.c_int64 * 3)()
        check(_lib.load().GB300TessellationCount(
            self.regular_face_size, self.num_faces, _ptr(self.face_sizes),
            _ptr(self.rate_offsets), _ptr(self.rates), self.uniform_rate, C.byref(self.options),
            _ptr(self.coord_offsets), _ptr(self.facet_offsets), _ptr(self.ptex_offsets), totals,
            _stream(self.stream)))
        self.num_coords, self.num_facets, self.num_ptex_faces = (int(x) for x in totals)
        return self.num_coords, self.num_facets

    @property
    def coord_stride(self):
        return self.options.coordStride or 2

    @property
    def facet_stride(self):
        return self.options.facetStride or self.options.GetFacetSize()

    def Generate(self, coords=None, facets=None, offset_facet_indices=True, table=None,
                 patch_coords=None):
        """Writes coords [num_coords, coord_stride] float32 and facets
        [num_facets, facet_stride] int32 (allocated when not given), and with a
        GB300PatchTable the PatchCoords [num_coords, 5] int32 of every coord.  Returns
        (coords, facets, patch_coords)."""
        torch = _torch()
        dev = torch.device("cuda")
        if coords is None:
            coords = torch.zeros((self.num_coords, self.coord_stride), dtype=torch.float32,
                                 device=dev)
        if facets is None:
            facets = torch.zeros((self.num_facets, self.facet_stride), dtype=torch.int32,
                                 device=dev)
        if table is not None and patch_coords is None:
            patch_coords = torch.zeros((self.num_coords, 5), dtype=torch.int32, device=dev)
        check(_lib.load().GB300TessellationGenerate(
            self.regular_face_size, self.num_faces, _ptr(self.face_sizes),
            _ptr(self.rate_offsets), _ptr(self.rates), self.uniform_rate, C.byref(self.options),
            _ptr(self.coord_offsets), _ptr(self.facet_offsets), _ptr(self.ptex_offsets),
            _ptr(coords), _ptr(facets), int(bool(offset_facet_indices)),
            table.handle if table is not None else None,
            _ptr(patch_coords) if table is not None else None, _stream(self.stream)))
        return coords, facets, patch_coords

    def Share(self, face_verts, face_edges, num_vertices, num_edges, facets,
              patch_coords=None, coords=None, mesh_facet_indices=True, point_coords=False,
              point_faces=False, vertex_points=False, edge_points=False, out=None):
        """Shared (watertight) points, as the reference's Bfr tutorial 2.2 shares vertex and
        edge points (GB300TessellationShare): face_verts / face_edges are the base level's
        face vertices and edges per corner (host arrays or CUDA tensors); `facets` from
        Generate (mesh-wide indices unless mesh_facet_indices is False) are rewritten in place
        to point indices.  Returns a SharedPoints: num_points, point_offsets [faces + 1] and,
        as asked, patch_coords [num_points, 5] (copied from the coords' `patch_coords`: give
        them to Evaluate with num_points), coords [num_points, 2], faces, vertex_points,
        edge_points.  `out`: a SharedPoints from an earlier call on the same mesh, whose
        buffers are reused (nothing is allocated)."""
        torch = _torch()
        dev = torch.device("cuda")

        def on_device(x):
            t = x if hasattr(x, "data_ptr") else torch.from_numpy(np.ascontiguousarray(x, np.int32))
            return t.to(dev, torch.int32).contiguous()

        fv, fe = on_device(face_verts), on_device(face_edges)
        if point_coords and coords is None:
            raise ValueError("point_coords needs the tessellation's coords")
        if out is None:
            cap = max(self.num_coords, 1)
            out = SharedPoints()
            out.point_offsets = torch.empty(self.num_faces + 1, dtype=torch.int64, device=dev)
            out._pc = (torch.empty((cap, 5), dtype=torch.int32, device=dev)
                       if patch_coords is not None else None)
            out._coords = (torch.empty((cap, 2), dtype=torch.float32, device=dev)
                           if point_coords else None)
            out._faces = (torch.empty(cap, dtype=torch.int32, device=dev)
                          if point_faces else None)
            out.vertex_points = (torch.empty(max(int(num_vertices), 1), dtype=torch.int32,
                                             device=dev) if vertex_points else None)
            out.edge_points = (torch.empty(max(int(num_edges), 1), dtype=torch.int32,
                                           device=dev) if edge_points else None)
        elif ((patch_coords is not None and out._pc is None) or
              (point_coords and out._coords is None) or (point_faces and out._faces is None)):
            raise ValueError("`out` lacks a buffer this call writes")
        n = C.c_int64(0)
        check(_lib.load().GB300TessellationShare(
            self.regular_face_size, self.num_faces, _ptr(self.face_sizes),
            _ptr(self.rate_offsets), _ptr(self.rates), self.uniform_rate, C.byref(self.options),
            _ptr(self.coord_offsets), _ptr(self.facet_offsets), _ptr(fv), _ptr(fe),
            int(fv.numel()), int(num_vertices), int(num_edges), _ptr(facets),
            int(bool(mesh_facet_indices)),
            _ptr(patch_coords), _ptr(coords), _ptr(out.point_offsets),
            _ptr(out._pc if patch_coords is not None else None),
            _ptr(out._coords if point_coords else None),
            _ptr(out._faces if point_faces else None), _ptr(out.vertex_points),
            _ptr(out.edge_points), C.byref(n), _stream(self.stream)))
        out.num_points = np_ = int(n.value)
        out.patch_coords = out._pc[:np_] if patch_coords is not None else None
        out.coords = out._coords[:np_] if point_coords else None
        out.faces = out._faces[:np_] if point_faces else None
        return out

    def Evaluate(self, src, src_desc, table, patch_coords, derivatives=1, outputs=None,
                 num_points=None):
        """Limit points at every coord (Bfr::Surface::Evaluate, GB300TessellationEvaluate): P,
        and with derivatives >= 1 Du, Dv, with 2 also Duu, Duv, Dvv; each [n, length] float32
        (allocated unless `outputs` gives them), n = num_coords, or num_points for the shared
        points of Share."""
        torch = _torch()
        n = self.num_coords if num_points is None else int(num_points)
        L = src_desc.length
        k = 1 if derivatives == 0 else 3 if derivatives == 1 else 6
        outs = outputs if outputs is not None else [
            torch.zeros((n, L), dtype=torch.float32, device="cuda") for _ in range(k)]
        ptrs = [_ptr(outs[i]) if i < k else None for i in range(6)]
        check(_lib.load().GB300TessellationEvaluate(
            table.handle, _ptr(src, src_desc.offset), *ptrs, L, src_desc.stride, *([L] * 6), n,
            _ptr(patch_coords), _stream(self.stream)))
        return outs[:k]


    def EvaluateVarying(self, src, src_desc, table, patch_coords, derivatives=0, outputs=None,
                        num_points=None):
        """Varying values at every coord (the linear surfaces of
        Bfr::SurfaceFactory::InitVaryingSurface, bfr/surfaceFactory.h:252): `table`'s varying
        patches (GB300PatchTable.SetVarying, or Create from a Far table) at the coords'
        PatchCoords, over `src` holding the varying values of the control vertices and of the
        refined vertices (Far::StencilTableFactory in INTERPOLATE_VARYING mode) --
        GB300PatchTableEvalVarying; value, and with derivatives >= 1 d/du and d/dv, each
        [n, length] float32."""
        torch = _torch()
        n = self.num_coords if num_points is None else int(num_points)
        L = src_desc.length
        k = 1 if derivatives == 0 else 3
        outs = outputs if outputs is not None else [
            torch.zeros((n, L), dtype=torch.float32, device="cuda") for _ in range(k)]
        ptrs = [_ptr(outs[i]) if i < k else None for i in range(6)]
        check(_lib.load().GB300PatchTableEvalVarying(
            table.handle, _ptr(src, src_desc.offset), *ptrs, L, src_desc.stride, *([L] * 6), n,
            _ptr(patch_coords), _stream(self.stream)))
        return outs[:k]

    def EvaluateFaceVarying(self, src, src_desc, table, patch_coords, channel=0, derivatives=0,
                            outputs=None):
        """Face-varying values at every coord (the face-varying surfaces of
        Bfr::SurfaceFactory::InitFaceVaryingSurface): channel `channel` of `table` evaluated at
        the coords' PatchCoords (GB300PatchTableEvalFaceVarying); value, and with
        derivatives >= 1 d/du and d/dv, each [num_coords, length] float32."""
        torch = _torch()
        n = self.num_coords
        L = src_desc.length
        k = 1 if derivatives == 0 else 3
        outs = outputs if outputs is not None else [
            torch.zeros((n, L), dtype=torch.float32, device="cuda") for _ in range(k)]
        ptrs = [_ptr(outs[i]) if i < k else None for i in range(6)]
        check(_lib.load().GB300PatchTableEvalFaceVarying(
            table.handle, int(channel), _ptr(src, src_desc.offset), *ptrs, L, src_desc.stride,
            *([L] * 6), n, _ptr(patch_coords), _stream(self.stream)))
        return outs[:k]


class Tessellation:
    """Bfr::Tessellation of one face (its pattern is computed on the device)."""

    def __init__(self, param: Parameterization, rates, options=None):
        rates = np.atleast_1d(np.asarray(rates, np.int32))
        self._param = param
        self._rates = rates
        self._options = options if options is not None else TessellationOptions()
        size = param.GetFaceSize() if param.IsValid() else 0
        self._mesh = MeshTessellation(param.regular_face_size, np.array([size], np.int32),
                                      rates=rates, rate_offsets=np.array([0, len(rates)], np.int32),
                                      options=self._options)
        self._coords = self._facets = None

    def IsValid(self) -> bool: return self._mesh.num_coords > 0
    def GetParameterization(self) -> Parameterization: return self._param
    def GetFaceSize(self) -> int: return self._param.GetFaceSize()
    def GetNumCoords(self) -> int: return self._mesh.num_coords
    def GetNumFacets(self) -> int: return self._mesh.num_facets
    def GetFacetSize(self) -> int: return self._options.GetFacetSize()

    def _generate(self):
        if self._coords is None:
            c, f, _ = self._mesh.Generate(offset_facet_indices=False)
            _torch().cuda.synchronize()
            self._coords = c.cpu().numpy()
            self._facets = f.cpu().numpy()

    def GetCoords(self) -> np.ndarray:
        """[GetNumCoords(), coord stride] float32: boundary coords first, then interior."""
        self._generate()
        return self._coords

    def GetFacets(self) -> np.ndarray:
        """[GetNumFacets(), facet stride] int32 coord indices (-1 pads a triangle in a 4-tuple)."""
        self._generate()
        return self._facets
