"""ctypes wrapper over oracle/_build/liboracle.so (the C restatement in osd_oracle.c).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU baseline are
the only callers.  The product path never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(quiet=True) -> str:
    """Compile liboracle.so with oracle/Makefile (gcc, a second or two)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _lib.orc_patchmap_build.restype = C.c_void_p
        _lib.orc_patchmap_free.argtypes = [C.c_void_p]
        _lib.orc_find_patches.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p]
        _lib.orc_patch_basis_f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                                           C.c_void_p]
        _lib.orc_patch_basis_d.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                           C.c_void_p]
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _ptrs(arrs):
    return (C.c_void_p * len(arrs))(*[(a.ctypes.data if a is not None else None) for a in arrs])


def eval_stencils(src, src_desc, dsts, dst_descs, sizes, offsets, indices, weights,
                  start=0, end=None, threads=1, fp64=False):
    """Restated EvalStencils (osd/cpuKernel.cpp:71-240).  dsts are float32 (or float64 when
    fp64) arrays, written at absolute stencil positions i in [start, end)."""
    if end is None:
        end = len(sizes)
    fn = lib().orc_eval_stencils_d if fp64 else lib().orc_eval_stencils_f
    ok = fn(_p(np.ascontiguousarray(src, np.float32)), _p(np.asarray(src_desc, np.int32)),
            C.c_int(len(dsts)), _ptrs(dsts), _p(np.asarray(dst_descs, np.int32).ravel()),
            _p(sizes), _p(offsets), _p(indices), _ptrs(weights), C.c_int(start), C.c_int(end),
            C.c_int(threads))
    return bool(ok)


def eval_patches(src, src_desc, dsts, dst_descs, coords, arrays, indices, params, threads=1,
                 fp64=False, absolute=False):
    """Restated EvalPatches (osd/cpuEvaluator.cpp:157-381).  coords: int32 [n, 5] view of
    PatchCoord records (s, t stored as float bits).  absolute=True writes sum_j |w_j x_j|
    (double) instead: the scale of the float rounding error of each output."""
    if absolute:
        fn = lib().orc_eval_patches_abs
    else:
        fn = lib().orc_eval_patches_d if fp64 else lib().orc_eval_patches_f
    ok = fn(_p(np.ascontiguousarray(src, np.float32)), _p(np.asarray(src_desc, np.int32)),
            C.c_int(len(dsts)), _ptrs(dsts), _p(np.asarray(dst_descs, np.int32).ravel()),
            C.c_int(coords.shape[0]), _p(coords), _p(arrays), _p(indices), _p(params),
            C.c_int(threads))
    return bool(ok)


def abs_scale(src, src_desc, length, coords, arrays, indices, params):
    """[6, n*length] array of sum_j |w_j x_j| for the six EvalPatches outputs."""
    m = coords.shape[0]
    outs = [np.zeros(m * length) for _ in range(6)]
    eval_patches(src, src_desc, outs, [(0, length, length)] * 6, coords, arrays, indices, params,
                 threads=4, absolute=True)
    return np.stack(outs)


def stencil_abs_scale(src, src_desc, sizes, offsets, indices, weights, threads=4):
    """sum_j |w_j x_j| per stencil and element (double), for tolerance statements."""
    n = len(sizes)
    length = src_desc[1]
    out = np.zeros(n * length)
    eval_stencils(np.abs(np.asarray(src, np.float32)), src_desc, [out], [(0, length, length)],
                  sizes, offsets, indices, [np.abs(np.asarray(weights, np.float32))],
                  threads=threads, fp64=True)
    return out


def patch_basis(ptype, field0, field1, s, t, fp64=False):
    """Weights [6, n] of one point (osd/patchBasis.h:1558-1610)."""
    w = np.zeros(120, np.float64 if fp64 else np.float32)
    fn = lib().orc_patch_basis_d if fp64 else lib().orc_patch_basis_f
    n = fn(ptype, int(np.int32(field0)), int(np.int32(field1)), s, t, _p(w))
    return w.reshape(6, 20)[:, :n]


def patch_masks(coords, arrays, indices, params, channels=3):
    """Per-point masks of limit stencils at PatchCoords (int32 [n, 5]): the patch's control
    points and their basis weights (patch_basis), as Far::LimitStencilTableFactory merges them
    over its point stencils (far/stencilTableFactory.cpp:560-640).  Returns (offsets [n + 1],
    sources, [weights per channel]) for compose_rows; a point without a patch gets no entries."""
    c = np.asarray(coords, np.int32).reshape(-1, 5)
    arrays = np.asarray(arrays, np.int32).reshape(-1, 6)
    indices = np.asarray(indices, np.int32)
    params = np.asarray(params, np.int32).reshape(-1, 3)
    st = c[:, 3:5].copy().view(np.float32)
    offs, src, ws = [0], [], [[] for _ in range(channels)]
    for i in range(len(c)):
        a, pi = int(c[i, 0]), int(c[i, 1])
        if a < 0:
            offs.append(offs[-1])
            continue
        reg, desc, _, ib, stride, pb = (int(x) for x in arrays[a])
        f0, f1 = int(params[pi, 0]), int(params[pi, 1])
        ptype = reg if (f1 >> 5) & 1 else desc
        w = patch_basis(ptype, f0, f1, float(st[i, 0]), float(st[i, 1]))
        n = w.shape[1]
        src.extend(indices[ib + stride * (pi - pb): ib + stride * (pi - pb) + n])
        for k in range(channels):
            ws[k].extend(w[k])
        offs.append(offs[-1] + n)
    return (np.asarray(offs, np.int64), np.asarray(src, np.int32),
            [np.asarray(w, np.float32) for w in ws])


class PatchMap:
    """Restated Far::PatchMap (far/patchMap.cpp)."""

    def __init__(self, arrays, params, triangular):
        self.arrays = np.ascontiguousarray(arrays, np.int32)
        self.params = np.ascontiguousarray(params, np.int32)
        self.h = C.c_void_p(lib().orc_patchmap_build(C.c_int(len(self.arrays)), _p(self.arrays),
                                                     _p(self.params), C.c_int(int(triangular))))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_patchmap_free(self.h)
            self.h = None

    def find(self, faces, u, v):
        faces = np.ascontiguousarray(faces, np.int32)
        u = np.ascontiguousarray(u, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        out = np.zeros((len(faces), 3), np.int32)
        lib().orc_find_patches(self.h, len(faces), _p(faces), _p(u), _p(v), _p(out))
        return out


def make_coords(handles, s, t):
    """Pack handles [n,3] + (s,t) float32 into int32 [n,5] PatchCoord records."""
    n = len(handles)
    out = np.zeros((n, 5), np.int32)
    out[:, :3] = handles
    out[:, 3] = np.asarray(s, np.float32).view(np.int32)
    out[:, 4] = np.asarray(t, np.float32).view(np.int32)
    return out


class _OrcTable(C.Structure):
    _fields_ = [("numStencils", C.c_int), ("numChannels", C.c_int), ("nnz", C.c_longlong),
                ("sizes", C.POINTER(C.c_int)), ("offsets", C.POINTER(C.c_int)),
                ("indices", C.POINTER(C.c_int)), ("w", C.POINTER(C.c_float) * 6)]


def _take_table(ptr):
    if not ptr:
        raise ValueError("malformed masks")
    t = ptr.contents
    n, nnz = t.numStencils, t.nnz
    out = dict(sizes=np.ctypeslib.as_array(t.sizes, (max(n, 1),))[:n].copy(),
               offsets=np.ctypeslib.as_array(t.offsets, (max(n, 1),))[:n].copy(),
               indices=np.ctypeslib.as_array(t.indices, (max(nnz, 1),))[:nnz].copy())
    names = ("weights", "du_weights", "dv_weights", "duu_weights", "duv_weights",
             "dvv_weights")
    for c in range(t.numChannels):
        out[names[c]] = np.ctypeslib.as_array(t.w[c], (max(nnz, 1),))[:nnz].copy()
    lib().orc_table_free(ptr)
    return out


def _factory_protos():
    L = lib()
    if getattr(L, "_factory_protos", False):
        return L
    L.orc_factory_create.restype = C.POINTER(_OrcTable)
    L.orc_compose_rows.restype = C.POINTER(_OrcTable)
    L.orc_table_free.argtypes = [C.POINTER(_OrcTable)]
    L._factory_protos = True
    return L


def factory_create(num_control, levels, intermediate=True, control=False):
    """Restated Far::StencilTableFactory::Create (factorized) from per-level masks
    (dicts of offsets int64, sources int32, weights float32), as far/stencilBuilder.cpp
    merges them.  Returns dict(sizes, offsets, indices, weights)."""
    L = _factory_protos()
    offs = [np.ascontiguousarray(d["offsets"], np.int64) for d in levels]
    srcs = [np.ascontiguousarray(d["sources"], np.int32) for d in levels]
    ws = [np.ascontiguousarray(d["weights"], np.float32) for d in levels]
    nrows = np.array([len(o) - 1 for o in offs], np.int32)
    ptr = L.orc_factory_create(
        C.c_int(num_control), C.c_int(len(offs)), _p(nrows), _ptrs(offs) if offs else None,
        _ptrs(srcs) if offs else None, _ptrs(ws) if offs else None,
        C.c_int(int(intermediate)), C.c_int(int(control)))
    return _take_table(ptr)


def compose_rows(base, offsets, sources, weights, append_base=False):
    """Restated StencilBuilder::Index::AddWithWeight(StencilReal, ...) composition of rows
    over a base table (dict of sizes, offsets, indices, weights); weights is a list of 1, 3
    or 6 float32 arrays (P, du, dv[, duu, duv, dvv])."""
    L = _factory_protos()
    bs = np.ascontiguousarray(base["sizes"], np.int32)
    bo = np.ascontiguousarray(base["offsets"], np.int32)
    bi = np.ascontiguousarray(base["indices"], np.int32)
    bw = np.ascontiguousarray(base["weights"], np.float32)
    off = np.ascontiguousarray(offsets, np.int64)
    src = np.ascontiguousarray(sources, np.int32)
    ws = [np.ascontiguousarray(w, np.float32) for w in weights]
    ptr = L.orc_compose_rows(C.c_int(len(bs)), _p(bs), _p(bo), _p(bi), _p(bw),
                             C.c_int(len(off) - 1), _p(off), _p(src), C.c_int(len(ws)),
                             _ptrs(ws), C.c_int(int(append_base)))
    return _take_table(ptr)


# ---- Bfr::Parameterization / Bfr::Tessellation restatement (bfr_oracle.c) -----------------

def param_to_subface(reg_face_size, face_size, uv):
    """Parameterization::ConvertCoordToNormalizedSubFace over [n, 2] float32 coords:
    (sub-face [n], normalized coords [n, 2])."""
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    sub = np.zeros(len(uv), np.int32)
    st = np.zeros_like(uv)
    if not lib().orc_param_to_subface(C.c_int(reg_face_size), C.c_int(face_size),
                                      C.c_int(len(uv)), _p(uv), _p(sub), _p(st)):
        raise ValueError("invalid parameterization")
    return sub, st


def tess_inventory(reg_face_size, face_size, rates, facet_size=3, preserve_quads=False):
    """(valid, coords, facets, boundary coords, uniform) of one Bfr::Tessellation."""
    rates = np.ascontiguousarray(np.atleast_1d(rates), np.int32)
    c = np.zeros(4, np.int32)
    ok = lib().orc_tess_inventory(C.c_int(reg_face_size), C.c_int(face_size), C.c_int(len(rates)),
                                  _p(rates), C.c_int(facet_size), C.c_int(int(preserve_quads)),
                                  _p(c))
    return bool(ok), int(c[0]), int(c[1]), int(c[2]), bool(c[3])


def tess_generate(reg_face_size, face_size, rates, facet_size=3, preserve_quads=False):
    """(coords [n, 2] float32, facets [m, facet_size] int32) of one face, or None if invalid."""
    ok, nc, nf, _, _ = tess_inventory(reg_face_size, face_size, rates, facet_size,
                                      preserve_quads)
    if not ok:
        return None
    rates = np.ascontiguousarray(np.atleast_1d(rates), np.int32)
    coords = np.zeros((nc, 2), np.float32)
    fs = 4 if facet_size == 4 else 3
    facets = np.zeros((nf, fs), np.int32)
    r = lib().orc_tess_generate(C.c_int(reg_face_size), C.c_int(face_size), C.c_int(len(rates)),
                                _p(rates), C.c_int(fs), C.c_int(int(preserve_quads)), _p(coords),
                                C.c_int(2), _p(facets), C.c_int(fs))
    if r != 1:
        raise RuntimeError("tessellation restatement produced inconsistent counts")
    return coords, facets


def tess_mesh(reg_face_size, face_sizes, rate_offsets, rates, facet_size=3,
              preserve_quads=False, threads=1):
    """Every face of a mesh (Tessellation per face, facets offset to mesh-wide coords):
    dict(coord_offsets, facet_offsets, coords [n, 2], facets [m, facet_size])."""
    face_sizes = np.ascontiguousarray(face_sizes, np.int32)
    rate_offsets = np.ascontiguousarray(rate_offsets, np.int32)
    rates = np.ascontiguousarray(rates, np.int32)
    nfaces = len(face_sizes)
    counts = np.zeros((nfaces, 2), np.int64)
    c = np.zeros(4, np.int32)
    L = lib()
    for f in range(nfaces):
        r = rates[rate_offsets[f]:rate_offsets[f + 1]]
        L.orc_tess_inventory(C.c_int(reg_face_size), C.c_int(int(face_sizes[f])),
                             C.c_int(len(r)), _p(np.ascontiguousarray(r)), C.c_int(facet_size),
                             C.c_int(int(preserve_quads)), _p(c))
        counts[f] = c[:2]
    co = np.zeros(nfaces + 1, np.int64)
    fo = np.zeros(nfaces + 1, np.int64)
    co[1:] = np.cumsum(counts[:, 0])
    fo[1:] = np.cumsum(counts[:, 1])
    fs = 4 if facet_size == 4 else 3
    coords = np.zeros((int(co[-1]), 2), np.float32)
    facets = np.zeros((int(fo[-1]), fs), np.int32)
    ok = L.orc_tess_mesh(C.c_int(reg_face_size), C.c_int(nfaces), _p(face_sizes),
                         _p(rate_offsets), _p(rates), C.c_int(fs), C.c_int(int(preserve_quads)),
                         _p(co), _p(fo), _p(coords), _p(facets), C.c_int(threads))
    if not ok:
        raise RuntimeError("tessellation restatement produced inconsistent counts")
    return dict(coord_offsets=co, facet_offsets=fo, coords=coords, facets=facets)


def tess_locate_mesh(reg_face_size, face_sizes, coord_offsets, ptex_offsets, coords, threads=1):
    """(ptex faces [n], (s, t) [n, 2]) of every coord of a mesh tessellation."""
    face_sizes = np.ascontiguousarray(face_sizes, np.int32)
    co = np.ascontiguousarray(coord_offsets, np.int64)
    po = np.ascontiguousarray(ptex_offsets, np.int64)
    coords = np.ascontiguousarray(coords, np.float32).reshape(-1, 2)
    faces = np.zeros(len(coords), np.int32)
    st = np.zeros_like(coords)
    if not lib().orc_tess_locate_mesh(C.c_int(reg_face_size), C.c_int(len(face_sizes)),
                                      _p(face_sizes), _p(co), _p(po), _p(coords), _p(faces),
                                      _p(st), C.c_int(threads)):
        raise ValueError("invalid parameterization in the mesh")
    return faces, st


def tess_share(reg_face_size, face_sizes, face_verts, face_edges, num_vertices, num_edges,
               rate_offsets, rates, coord_offsets, facet_offsets, facets, facet_size=3,
               preserve_quads=False, mesh_indices=True):
    """Shared (watertight) points of a mesh tessellation (the reference's tutorial 2.2
    bookkeeping): (facets rewritten to point indices, point_offsets [faces + 1],
    point_sources [points] = the mesh coord each point was made from)."""
    face_sizes = np.ascontiguousarray(face_sizes, np.int32)
    fv = np.ascontiguousarray(face_verts, np.int32)
    fe = np.ascontiguousarray(face_edges, np.int32)
    ro = np.ascontiguousarray(rate_offsets, np.int32)
    rates = np.ascontiguousarray(rates, np.int32)
    co = np.ascontiguousarray(coord_offsets, np.int64)
    fo = np.ascontiguousarray(facet_offsets, np.int64)
    fs = 4 if facet_size == 4 else 3
    out = np.array(facets, np.int32, copy=True).reshape(-1, fs)
    nf = len(face_sizes)
    po = np.zeros(nf + 1, np.int64)
    src = np.zeros(max(int(co[-1]), 1), np.int64)
    L = lib()
    L.orc_tess_share.restype = C.c_long
    n = L.orc_tess_share(C.c_int(reg_face_size), C.c_int(nf), _p(face_sizes), _p(fv), _p(fe),
                         C.c_int(num_vertices), C.c_int(num_edges), _p(ro), _p(rates),
                         C.c_int(fs), C.c_int(int(preserve_quads)), _p(co), _p(fo), C.c_int(fs),
                         C.c_int(int(mesh_indices)), _p(out), _p(po), _p(src))
    if n < -nf:
        raise ValueError("vertex or edge index out of range")
    if n < 0:
        raise ValueError(f"face {-1 - n} runs a shared edge at another rate")
    return out, po, src[:n]


def edge_numbering(face_sizes, face_verts):
    """One index per undirected edge (numbered in order of first appearance) for every face
    corner -- the edge from corner i to corner i + 1 -- and the number of edges.  Any
    consistent numbering gives the same shared points."""
    face_sizes = np.asarray(face_sizes, np.int64)
    fv = np.asarray(face_verts, np.int64)
    start = np.concatenate([[0], np.cumsum(face_sizes)])
    nxt = np.arange(len(fv)) + 1
    last = start[1:] - 1
    nxt[last[face_sizes > 0]] = start[:-1][face_sizes > 0]
    a, b = fv, fv[nxt] if len(fv) else fv
    key = np.minimum(a, b) * (int(fv.max(initial=0)) + 1) + np.maximum(a, b)
    _, first, inv = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(np.argsort(first))
    return order[inv].astype(np.int32), len(first)


# ---- draw-time tessellation factors (tess_factors_oracle.c) --------------------------------

def tess_factors(arrays, indices, params, src, src_stride, tess_level, max_tess_level=64.0,
                 screen_space=False, spacing=0, model_view=None, projection=None):
    """Per-patch (outer [n, 4], inner [n, 2], lo [n, 4], hi [n, 4]) of the patch shaders'
    tess-control math (osd/glslPatchCommonTess.glsl:92-550)."""
    arrays = np.ascontiguousarray(arrays, np.int32)
    indices = np.ascontiguousarray(indices, np.int32)
    params = np.ascontiguousarray(params, np.int32)
    n = len(params)
    mv = np.ascontiguousarray(model_view if model_view is not None else np.eye(4), np.float32)
    pr = np.ascontiguousarray(projection if projection is not None else np.eye(4), np.float32)
    outs = [np.zeros((n, 4), np.float32), np.zeros((n, 2), np.float32),
            np.zeros((n, 4), np.float32), np.zeros((n, 4), np.float32)]
    srcp = np.ascontiguousarray(src, np.float32) if src is not None else None
    lib().orc_tess_factors(_p(arrays), C.c_int(len(arrays)), _p(indices), _p(params), C.c_int(n),
                           _p(srcp), C.c_int(src_stride), C.c_float(tess_level),
                           C.c_float(max_tess_level), C.c_int(int(screen_space)),
                           C.c_int(spacing), _p(mv.T.copy()), _p(pr.T.copy()),
                           *[_p(o) for o in outs])
    return tuple(outs)


def tess_parameterization(domain, patch_index, lo, hi, spacing=0, triangular=False):
    """OsdGetTessParameterization[Triangle]: patch (u, v) [n, 2] of domain points [n, 3]."""
    domain = np.ascontiguousarray(domain, np.float32).reshape(-1, 3)
    patch_index = np.ascontiguousarray(patch_index, np.int32)
    uv = np.zeros((len(domain), 2), np.float32)
    lib().orc_tess_parameterization(C.c_int(len(domain)), _p(domain), _p(patch_index),
                                    _p(np.ascontiguousarray(lo, np.float32)),
                                    _p(np.ascontiguousarray(hi, np.float32)), C.c_int(spacing),
                                    C.c_int(int(triangular)), _p(uv))
    return uv
