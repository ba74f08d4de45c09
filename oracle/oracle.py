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
