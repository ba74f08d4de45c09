"""ctypes wrapper over oracle/_ref/libosdref.so: the reference's own Far/Osd CPU code.

TEST INFRASTRUCTURE ONLY.  Available where the reference sources were present to compile
(``make -C oracle ref``); used to generate golden fixtures and to cross-check the oracle.
Nothing in the product imports this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libosdref.so")

_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        _lib.ref_refiner_create.restype = vp
        _lib.ref_refiner_create_fvar.restype = vp
        _lib.ref_stencils_create.restype = vp
        _lib.ref_limit_stencils_create.restype = vp
        _lib.ref_patches_create.restype = vp
        _lib.ref_stencils_nnz.restype = C.c_long
        _lib.ref_stencils_create_mode.restype = vp
        _lib.ref_masks_record.restype = vp
        _lib.ref_limit_record.restype = vp
        _lib.ref_limit_array_size.restype = C.c_long
        for name in ("ref_refiner_destroy", "ref_refine_uniform", "ref_refine_adaptive",
                     "ref_num_vertices_total", "ref_level_num_vertices", "ref_max_level",
                     "ref_num_ptex_faces", "ref_ptex_face_ids", "ref_stencils_num",
                     "ref_stencils_nnz", "ref_stencils_num_control", "ref_stencils_copy",
                     "ref_stencils_destroy", "ref_patches_destroy", "ref_patches_counts",
                     "ref_patches_copy", "ref_patches_copy_stencils", "ref_find_patches",
                     "ref_cpu_eval_stencils", "ref_cpu_eval_patches", "ref_eval_patches_fp64",
                     "ref_omp_set_threads", "ref_patches_varying", "ref_patches_fvar",
                     "ref_masks_num_levels", "ref_masks_num_control", "ref_masks_level_counts",
                     "ref_masks_level_copy", "ref_masks_destroy", "ref_limit_array_size",
                     "ref_limit_array_copy", "ref_limit_info", "ref_limit_destroy"):
            getattr(_lib, name).argtypes = None
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Refiner:
    """Far::TopologyRefiner built from a shapes.Cage (far/topologyRefinerFactory.h)."""

    def __init__(self, cage, boundary: int = 1, fvar=None):
        """fvar: optional (num_values, value index per face-vertex, linear) face-varying
        channel."""
        self.cage = cage
        L = lib()
        cv = np.ascontiguousarray(cage.crease_verts, np.int32).ravel()
        cs = np.ascontiguousarray(cage.crease_sharpness, np.float32)
        # optional vertex (corner) sharpness and boundary interpolation of the cage
        kv = np.ascontiguousarray(getattr(cage, "corner_verts", np.zeros(0)), np.int32)
        ks = np.ascontiguousarray(getattr(cage, "corner_sharpness", np.zeros(0)), np.float32)
        boundary = int(getattr(cage, "boundary", boundary))
        self._keep = (cage.verts_per_face, cage.face_verts, cv, cs, kv, ks)
        if fvar is None:
            self.h = L.ref_refiner_create(
                C.c_int(cage.scheme), C.c_int(cage.num_vertices), C.c_int(cage.num_faces),
                _p(cage.verts_per_face), _p(cage.face_verts), C.c_int(len(cs)), _p(cv), _p(cs),
                C.c_int(len(ks)), _p(kv) if len(ks) else None, _p(ks) if len(ks) else None,
                C.c_int(boundary))
        else:
            nvals, fidx, linear = fvar
            fidx = np.ascontiguousarray(fidx, np.int32)
            self._keep += (fidx,)
            self.h = L.ref_refiner_create_fvar(
                C.c_int(cage.scheme), C.c_int(cage.num_vertices), C.c_int(cage.num_faces),
                _p(cage.verts_per_face), _p(cage.face_verts), C.c_int(len(cs)), _p(cv), _p(cs),
                C.c_int(boundary), C.c_int(nvals), _p(fidx), C.c_int(int(bool(linear))))
        if not self.h:
            raise RuntimeError("TopologyRefinerFactory::Create failed")
        self.h = C.c_void_p(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_refiner_destroy(self.h)
            self.h = None

    def refine_uniform(self, level):
        lib().ref_refine_uniform(self.h, C.c_int(level))
        return self

    def refine_adaptive(self, level, single_crease=False, inf_sharp=False):
        lib().ref_refine_adaptive(self.h, C.c_int(level), C.c_int(int(single_crease)),
                                  C.c_int(int(inf_sharp)))
        return self

    def refine_adaptive_levels(self, primary, secondary, inf_sharp=True):
        """Adaptive refinement with a secondary level for smooth features, as the reference's
        Bfr regression refines the tables it compares Bfr::Surface against."""
        lib().ref_refine_adaptive_levels(self.h, C.c_int(primary), C.c_int(secondary),
                                         C.c_int(int(inf_sharp)))
        return self

    def num_vertices_total(self):
        return lib().ref_num_vertices_total(self.h)

    def level_num_vertices(self, level):
        return lib().ref_level_num_vertices(self.h, C.c_int(level))

    def num_ptex_faces(self):
        return lib().ref_num_ptex_faces(self.h)

    def ptex_face_ids(self):
        out = np.zeros(self.cage.num_faces, np.int32)
        lib().ref_ptex_face_ids(self.h, _p(out))
        return out


def _copy_stencils(h, limit, use_double):
    L = lib()
    n = L.ref_stencils_num(h)
    nnz = L.ref_stencils_nnz(h)
    wt = np.float64 if use_double else np.float32
    sizes = np.zeros(n, np.int32)
    offsets = np.zeros(n, np.int32)
    idx = np.zeros(nnz, np.int32)
    ws = [np.zeros(nnz, wt) for _ in range(6 if limit else 1)]
    arr = (C.c_void_p * 6)(*([w.ctypes.data for w in ws] + [None] * (6 - len(ws))))
    L.ref_stencils_copy(h, _p(sizes), _p(offsets), _p(idx), arr)
    out = dict(sizes=sizes, offsets=offsets, indices=idx, weights=ws[0],
               num_control=L.ref_stencils_num_control(h))
    if limit:
        for k, name in enumerate(("du", "dv", "duu", "duv", "dvv"), 1):
            out[name + "_weights"] = ws[k]
    L.ref_stencils_destroy(h)
    return out


def stencil_table(refiner, use_double=False, intermediate=True, factorize=True,
                  control=False, max_level=10):
    """Far::StencilTableFactoryReal<REAL>::Create (far/stencilTableFactory.cpp:78-151)."""
    h = C.c_void_p(lib().ref_stencils_create(refiner.h, C.c_int(int(use_double)),
                                             C.c_int(int(intermediate)), C.c_int(int(factorize)),
                                             C.c_int(int(control)), C.c_int(max_level)))
    return _copy_stencils(h, False, use_double)


INTERPOLATE_VERTEX, INTERPOLATE_VARYING, INTERPOLATE_FACE_VARYING = 0, 1, 2


def stencil_table_mode(refiner, mode=INTERPOLATE_VERTEX, channel=0, intermediate=True,
                       control=False, max_level=10):
    """Far::StencilTableFactory::Create (float) in interpolation mode `mode`."""
    h = C.c_void_p(lib().ref_stencils_create_mode(refiner.h, C.c_int(mode), C.c_int(channel),
                                                  C.c_int(int(intermediate)),
                                                  C.c_int(int(control)), C.c_int(max_level)))
    return _copy_stencils(h, False, False)


def record_masks(refiner, mode=INTERPOLATE_VERTEX, channel=0, max_level=10):
    """Per-level masks recorded from Far::PrimvarRefiner by the product's GB300MaskRecorder:
    (num_control, [dict(offsets int64, sources int32, weights float32), ...])."""
    L = lib()
    h = L.ref_masks_record(refiner.h, C.c_int(mode), C.c_int(channel), C.c_int(max_level))
    if not h:
        raise RuntimeError("mask recording failed")
    h = C.c_void_p(h)
    levels = []
    for lv in range(L.ref_masks_num_levels(h)):
        n, nnz = C.c_int(), C.c_long()
        L.ref_masks_level_counts(h, C.c_int(lv), C.byref(n), C.byref(nnz))
        off = np.zeros(n.value + 1, np.int64)
        src = np.zeros(nnz.value, np.int32)
        w = np.zeros(nnz.value, np.float32)
        L.ref_masks_level_copy(h, C.c_int(lv), _p(off), _p(src), _p(w))
        levels.append(dict(offsets=off, sources=src, weights=w))
    nc = L.ref_masks_num_control(h)
    L.ref_masks_destroy(h)
    return nc, levels


def limit_record(refiner, ptex, s, t, mode=INTERPOLATE_VERTEX, channel=0, d1=True, d2=False):
    """Inputs and outputs of the GPU limit-stencil factory for these locations, recorded with
    GB300LimitStencilTableFactory's helpers, plus Far::LimitStencilTableFactory's own table."""
    L = lib()
    ptex = np.ascontiguousarray(ptex, np.int32)
    s = np.ascontiguousarray(s, np.float32)
    t = np.ascontiguousarray(t, np.float32)
    h = L.ref_limit_record(refiner.h, C.c_int(mode), C.c_int(channel), C.c_int(len(ptex)),
                           _p(ptex), _p(s), _p(t), C.c_int(int(d1)), C.c_int(int(d2)))
    if not h:
        raise RuntimeError("limit recording failed")
    h = C.c_void_p(h)
    types = {0: np.int32, 1: np.int64, 2: np.int32, 3: np.float32, 4: np.int64, 5: np.int32,
             6: np.float32, 7: np.int64, 8: np.int32, 15: np.int32, 16: np.int32, 17: np.int32}
    names = {0: "level_rows", 1: "level_offsets", 2: "level_sources", 3: "level_weights",
             4: "local_offsets", 5: "local_sources", 6: "local_weights", 7: "loc_offsets",
             8: "loc_sources", 15: "far_sizes", 16: "far_offsets", 17: "far_indices"}
    out = {}
    for key in range(24):
        typ = types.get(key, np.float32)
        name = names.get(key, f"loc_w{key - 9}" if key < 15 else f"far_w{key - 18}")
        a = np.zeros(L.ref_limit_array_size(h, C.c_int(key)), typ)
        if len(a):
            L.ref_limit_array_copy(h, C.c_int(key), _p(a))
        out[name] = a
    info = np.zeros(4, np.int32)
    L.ref_limit_info(h, _p(info))
    out.update(num_control=int(info[0]), num_channels=int(info[1]), spliced=int(info[2]),
               cv_intermediate=int(info[3]))
    L.ref_limit_destroy(h)
    return out


def limit_stencil_table(refiner, ptex, s, t, use_double=False, d1=True, d2=False):
    """Far::LimitStencilTableFactoryReal<REAL>::Create (far/stencilTableFactory.cpp:411-662)."""
    ptex = np.ascontiguousarray(ptex, np.int32)
    s = np.ascontiguousarray(s, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    h = C.c_void_p(lib().ref_limit_stencils_create(refiner.h, C.c_int(int(use_double)),
                                                   C.c_int(len(ptex)), _p(ptex), _p(s), _p(t),
                                                   C.c_int(int(d1)), C.c_int(int(d2))))
    return _copy_stencils(h, True, use_double)


class Patches:
    """Far::PatchTable + Osd::CpuPatchTable flattening + Far::PatchMap."""

    ENDCAP_BILINEAR, ENDCAP_BSPLINE, ENDCAP_GREGORY = 1, 2, 3

    def __init__(self, refiner, endcap=3, max_isolation=10, single_crease=False,
                 inf_sharp=False, share_endcap_points=True, legacy_sharp_corners=True):
        L = lib()
        L.ref_patches_create_ex.restype = C.c_void_p
        self.h = C.c_void_p(L.ref_patches_create_ex(
            refiner.h, C.c_int(endcap), C.c_int(max_isolation), C.c_int(int(single_crease)),
            C.c_int(int(inf_sharp)), C.c_int(int(share_endcap_points)),
            C.c_int(int(legacy_sharp_corners))))
        counts = np.zeros(6, np.int64)
        L.ref_patches_counts(self.h, _p(counts))
        na, ni, npar, nloc, nst, nnz = (int(x) for x in counts)
        self.arrays = np.zeros((na, 6), np.int32)
        self.indices = np.zeros(ni, np.int32)
        self.params = np.zeros((npar, 3), np.int32)
        L.ref_patches_copy(self.h, _p(self.arrays), _p(self.indices), _p(self.params))
        self.num_local_points = nloc
        self.st = dict(sizes=np.zeros(nst, np.int32), offsets=np.zeros(nst, np.int32),
                       indices=np.zeros(nnz, np.int32), weights=np.zeros(nnz, np.float32))
        L.ref_patches_copy_stencils(self.h, _p(self.st["sizes"]), _p(self.st["offsets"]),
                                    _p(self.st["indices"]), _p(self.st["weights"]))

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_patches_destroy(self.h)
            self.h = None

    def varying(self):
        """(arrays [n, 6], indices) of Osd::CpuPatchTable's varying tables."""
        counts = np.zeros(2, np.int64)
        lib().ref_patches_varying(self.h, _p(counts), None, None)
        arrays = np.zeros((int(counts[0]), 6), np.int32)
        indices = np.zeros(int(counts[1]), np.int32)
        lib().ref_patches_varying(self.h, _p(counts), _p(arrays), _p(indices))
        return arrays, indices

    def fvar(self, channel=0):
        """(arrays [n, 6], indices, params [n, 3]) of face-varying channel `channel`."""
        counts = np.zeros(4, np.int64)
        lib().ref_patches_fvar(self.h, C.c_int(channel), _p(counts), None, None, None)
        arrays = np.zeros((int(counts[1]), 6), np.int32)
        indices = np.zeros(int(counts[2]), np.int32)
        params = np.zeros((int(counts[3]), 3), np.int32)
        lib().ref_patches_fvar(self.h, C.c_int(channel), _p(counts), _p(arrays), _p(indices),
                               _p(params))
        return arrays, indices, params

    def fvar_stencils(self, refiner, channel=0):
        """Stencils of face-varying channel `channel` over its base values: every refinement
        level, then the channel's local points (the source buffer of its patches)."""
        counts = np.zeros(2, np.int64)
        lib().ref_patches_fvar_stencils(refiner.h, self.h, C.c_int(channel), _p(counts), None,
                                        None, None, None)
        n, nnz = int(counts[0]), int(counts[1])
        st = dict(sizes=np.zeros(n, np.int32), offsets=np.zeros(n, np.int32),
                  indices=np.zeros(nnz, np.int32), weights=np.zeros(nnz, np.float32))
        lib().ref_patches_fvar_stencils(refiner.h, self.h, C.c_int(channel), _p(counts),
                                        _p(st["sizes"]), _p(st["offsets"]), _p(st["indices"]),
                                        _p(st["weights"]))
        return st

    def find_patches(self, faces, u, v):
        faces = np.ascontiguousarray(faces, np.int32)
        u = np.ascontiguousarray(u, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        handles = np.zeros((len(faces), 3), np.int32)
        found = np.zeros(len(faces), np.int32)
        lib().ref_find_patches(self.h, C.c_int(len(faces)), _p(faces), _p(u), _p(v),
                               _p(handles), _p(found))
        return handles, found

    def eval_fp64(self, src, length, stride, handles, s, t):
        """Far::PatchTable::EvaluateBasis<double> + double accumulation; [n, 6, length]."""
        n = len(handles)
        out = np.zeros((n, 6, length), np.float64)
        lib().ref_eval_patches_fp64(self.h, _p(np.ascontiguousarray(src, np.float32)),
                                    C.c_int(length), C.c_int(stride), C.c_int(n),
                                    _p(np.ascontiguousarray(handles, np.int32)),
                                    _p(np.ascontiguousarray(s, np.float64)),
                                    _p(np.ascontiguousarray(t, np.float64)), _p(out))
        return out


def _desc_arr(descs):
    return np.asarray(descs, np.int32).ravel()


def cpu_eval_stencils(src, src_desc, dsts, dst_descs, sizes, offsets, indices, weights,
                      start, end, omp=False):
    """Osd::CpuEvaluator / OmpEvaluator ::EvalStencils (osd/cpuEvaluator.cpp:37-125)."""
    nout = len(dsts)
    dp = (C.c_void_p * nout)(*[d.ctypes.data for d in dsts])
    wp = (C.c_void_p * nout)(*[w.ctypes.data for w in weights])
    sd = np.asarray(src_desc, np.int32)
    dd = _desc_arr(dst_descs)
    ok = lib().ref_cpu_eval_stencils(_p(src), _p(sd), C.c_int(nout), dp, _p(dd), _p(sizes),
                                     _p(offsets), _p(indices), wp, C.c_int(start), C.c_int(end),
                                     C.c_int(int(omp)))
    return bool(ok)


def cpu_eval_patches(src, src_desc, dsts, dst_descs, coords, arrays, indices, params):
    """Osd::CpuEvaluator::EvalPatches (osd/cpuEvaluator.cpp:157-381)."""
    nout = len(dsts)
    dp = (C.c_void_p * nout)(*[d.ctypes.data for d in dsts])
    sd = np.asarray(src_desc, np.int32)
    dd = _desc_arr(dst_descs)
    ok = lib().ref_cpu_eval_patches(_p(src), _p(sd), C.c_int(nout), dp, _p(dd),
                                    C.c_int(coords.shape[0]), _p(coords), _p(arrays),
                                    _p(indices), _p(params))
    return bool(ok)


def omp_set_threads(n):
    lib().ref_omp_set_threads(C.c_int(n))


# ---- Bfr ----------------------------------------------------------------------------------

def bfr_tess(reg_face_size, face_size, rates, facet_size=3, preserve_quads=False):
    """The reference's Bfr::Tessellation of one face: (counts {coords, facets, boundary,
    uniform}, coords [n, 2] float32, facets [m, facet_size]) or None when invalid."""
    rates = np.ascontiguousarray(np.atleast_1d(rates), np.int32)
    c = np.zeros(4, np.int32)
    L = lib()
    ok = L.ref_bfr_tess_counts(C.c_int(reg_face_size), C.c_int(face_size), C.c_int(len(rates)),
                               _p(rates), C.c_int(facet_size), C.c_int(int(preserve_quads)),
                               _p(c))
    if not ok:
        return None
    fs = 4 if facet_size == 4 else 3
    coords = np.zeros((int(c[0]), 2), np.float32)
    facets = np.zeros((int(c[1]), fs), np.int32)
    L.ref_bfr_tess(C.c_int(reg_face_size), C.c_int(face_size), C.c_int(len(rates)), _p(rates),
                   C.c_int(fs), C.c_int(int(preserve_quads)), _p(coords), _p(facets))
    return c.copy(), coords, facets


def bfr_subface(reg_face_size, face_size, uv):
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    sub = np.zeros(len(uv), np.int32)
    st = np.zeros_like(uv)
    if not lib().ref_bfr_subface(C.c_int(reg_face_size), C.c_int(face_size), C.c_int(len(uv)),
                                 _p(uv), _p(sub), _p(st)):
        return None
    return sub, st


def bfr_mesh_record(refiner, positions, rate_offsets, rates, facet_size=3, preserve_quads=False,
                    approx_sharp=6, approx_smooth=2, uvs=None):
    """Bfr tessellate-and-evaluate of every base face (the reference's tutorial loop):
    dict(coord_offsets, facet_offsets, valid, regular, coords, facets, f32 [6, n, 3],
    f64 [6, n, 3]); with `uvs` (values of face-varying channel 0, [m, 2]) also uv [3, n, 2]:
    UV, dUV/du, dUV/dv of the face-varying surfaces."""
    L = lib()
    L.ref_bfr_mesh_record.restype = C.c_void_p
    pos = np.ascontiguousarray(positions, np.float32)
    ro = np.ascontiguousarray(rate_offsets, np.int32)
    rt = np.ascontiguousarray(rates, np.int32)
    uv = np.ascontiguousarray(uvs, np.float32) if uvs is not None else None
    h = C.c_void_p(L.ref_bfr_mesh_record(refiner.h, C.c_int(approx_sharp),
                                         C.c_int(approx_smooth), _p(pos), _p(ro), _p(rt),
                                         C.c_int(facet_size), C.c_int(int(preserve_quads)),
                                         _p(uv)))
    try:
        sizes = np.zeros(3, np.int64)
        L.ref_bfr_record_sizes(h, _p(sizes))
        nf, nc, nfi = (int(x) for x in sizes)
        fs = 4 if facet_size == 4 else 3
        out = dict(coord_offsets=np.zeros(nf + 1, np.int64),
                   facet_offsets=np.zeros(nf + 1, np.int64),
                   valid=np.zeros(nf, np.int32), regular=np.zeros(nf, np.int32),
                   coords=np.zeros((nc, 2), np.float32),
                   facets=np.zeros((nfi // fs, fs), np.int32),
                   f32=np.zeros((6, nc, 3), np.float32), f64=np.zeros((6, nc, 3), np.float64))
        pf = (C.c_void_p * 6)(*[out["f32"][k].ctypes.data for k in range(6)])
        pd = (C.c_void_p * 6)(*[out["f64"][k].ctypes.data for k in range(6)])
        L.ref_bfr_record_copy(h, _p(out["coord_offsets"]), _p(out["facet_offsets"]),
                              _p(out["valid"]), _p(out["regular"]), _p(out["coords"]),
                              _p(out["facets"]), pf, pd)
        if uv is not None:
            out["uv"] = np.zeros((3, nc, 2), np.float32)
            pu = (C.c_void_p * 3)(*[out["uv"][k].ctypes.data for k in range(3)])
            L.ref_bfr_record_uv(h, pu)
        return out
    finally:
        L.ref_bfr_record_destroy(h)


def bfr_share(refiner, rate_offsets, rates, num_coords, num_facets, facet_size=3,
              preserve_quads=False, approx_sharp=6, approx_smooth=2):
    """The reference's tessellation with shared vertex and edge points (tutorial 2.2 loop):
    (facets [m, facet_size] of point indices, point_offsets [faces + 1], point_sources
    [points] = the coord of bfr_mesh_record's numbering each point is evaluated at)."""
    L = lib()
    L.ref_bfr_share.restype = C.c_long
    ro = np.ascontiguousarray(rate_offsets, np.int32)
    rt = np.ascontiguousarray(rates, np.int32)
    fs = 4 if facet_size == 4 else 3
    facets = np.zeros((num_facets, fs), np.int32)
    po = np.zeros(len(ro), np.int64)
    src = np.zeros(max(num_coords, 1), np.int64)
    n = L.ref_bfr_share(refiner.h, C.c_int(approx_sharp), C.c_int(approx_smooth), _p(ro),
                        _p(rt), C.c_int(fs), C.c_int(int(preserve_quads)), _p(facets), _p(po),
                        _p(src))
    if n < 0:
        raise ValueError("non-manifold or mismatched shared edge")
    return facets, po, src[:n]


def bfr_stencils(refiner, rate_offsets, rates, num_coords, facet_size=3, preserve_quads=False,
                 approx_sharp=6, approx_smooth=2):
    """Bfr::Surface::EvaluateStencil (P, Du, Dv) at every coord of the reference's tessellate
    loop, over mesh vertices: dict(sizes [coords], offsets [coords + 1], indices, wP, wDu, wDv)."""
    L = lib()
    L.ref_bfr_stencils.restype = C.c_long
    ro = np.ascontiguousarray(rate_offsets, np.int32)
    rt = np.ascontiguousarray(rates, np.int32)
    sizes = np.zeros(max(num_coords, 1), np.int32)
    args = (refiner.h, C.c_int(approx_sharp), C.c_int(approx_smooth), _p(ro), _p(rt),
            C.c_int(facet_size), C.c_int(int(preserve_quads)), C.c_long(num_coords))
    n = L.ref_bfr_stencils(*args, _p(sizes), C.c_long(0), None, None, None, None)
    if n < 0:
        raise ValueError("coord capacity")
    idx = np.zeros(max(n, 1), np.int32)
    w = [np.zeros(max(n, 1), np.float32) for _ in range(3)]
    m = L.ref_bfr_stencils(*args, _p(sizes), C.c_long(n), _p(idx), _p(w[0]), _p(w[1]), _p(w[2]))
    if m != n:
        raise ValueError("entry count changed between passes")
    sizes = sizes[:num_coords]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    return dict(sizes=sizes, offsets=off, indices=idx[:n], wP=w[0][:n], wDu=w[1][:n],
                wDv=w[2][:n])


def bfr_varying(refiner, rate_offsets, rates, num_coords, values, facet_size=3,
                preserve_quads=False, approx_sharp=6, approx_smooth=2):
    """Varying surfaces (SurfaceFactory::InitVaryingSurface) evaluated at every coord of the
    reference's tessellate loop: [coords, length] from `values` [vertices, length]."""
    L = lib()
    L.ref_bfr_varying.restype = C.c_long
    v = np.ascontiguousarray(values, np.float32)
    out = np.zeros((max(num_coords, 1), v.shape[1]), np.float32)
    n = L.ref_bfr_varying(refiner.h, C.c_int(approx_sharp), C.c_int(approx_smooth),
                          _p(np.ascontiguousarray(rate_offsets, np.int32)),
                          _p(np.ascontiguousarray(rates, np.int32)), C.c_int(facet_size),
                          C.c_int(int(preserve_quads)), _p(v), C.c_int(v.shape[1]), _p(out))
    if n != num_coords:
        raise ValueError(f"varying loop visited {n} coords, expected {num_coords}")
    return out[:num_coords]


def bfr_limit_rates(refiner, positions, num_corners, interval, max_rate, approx_sharp=6,
                    approx_smooth=2):
    """Tutorial 2.1's limit-option rates (one per face corner, 0 for faces without a surface)
    and the limit positions at the corners it measured ([corners, 3])."""
    rates = np.zeros(max(num_corners, 1), np.int32)
    pts = np.zeros((max(num_corners, 1), 3), np.float32)
    lib().ref_bfr_limit_rates(refiner.h, C.c_int(approx_sharp), C.c_int(approx_smooth),
                              _p(np.ascontiguousarray(positions, np.float32)),
                              C.c_float(interval), C.c_int(max_rate), _p(rates), _p(pts))
    return rates[:num_corners], pts[:num_corners]
