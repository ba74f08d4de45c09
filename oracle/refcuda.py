"""The reference's own CUDA evaluator kernels (osd/cudaKernel.cu), for timing and cross-checks.

Test and measurement infrastructure: `make -C oracle refcuda` compiles the device code of the
reference's cudaKernel.cu, from the file where it lies in the reference tree, into
oracle/_ref/osd_cudaKernel.cubin for sm_103a.  This module loads that cubin through the CUDA
driver API and launches its kernels with the reference's own launch logic:

* CudaEvalStencils (osd/cudaKernel.cu:351-383): length 3 at stride 3 ->
  computeStencilsNv<3, 256> on min(2048, ceil(n / 256)) blocks of 256; length 4 at stride 4 ->
  computeStencilsNv_v4<256> likewise; anything else -> the generic computeStencils<<<512, 32>>>;
* CudaEvaluator::EvalStencils with derivatives (osd/cudaEvaluator.cpp:171-292): one
  CudaEvalStencils per weight array;
* CudaEvalPatches / CudaEvalPatchesWithDerivatives (osd/cudaKernel.cu:387-424):
  computePatches<<<512, 32>>>.

Launches go on the current context's stream handle given by the caller (an int cudaStream_t).
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "osd_cudaKernel.cubin")

_NAMES = {
    "nv3": "_Z17computeStencilsNvILi3ELi256EEvPKfPfPKiS4_S4_S1_ii",
    "v4": "_Z20computeStencilsNv_v4ILi256EEvPKfPfPKiS4_S4_S1_ii",
    "generic": "_Z15computeStencilsPKfPfiiiPKiS3_S3_S0_ii",
    "patches": "_Z14computePatchesPKfPfS1_S1_S1_S1_S1_iiiiiiiiiPK13OsdPatchCoordPK13OsdPatchArray"
               "PKiPK13OsdPatchParam",
}

_mod = None
_fn = {}
_cu = None


def available() -> bool:
    return os.path.exists(CUBIN)


def _load():
    global _mod, _cu
    if _mod is not None:
        return
    _cu = C.CDLL("libcuda.so.1")
    mod = C.c_void_p()
    r = _cu.cuModuleLoad(C.byref(mod), CUBIN.encode())
    if r != 0:
        raise RuntimeError(f"cuModuleLoad({CUBIN}) failed: {r}")
    _mod = mod
    for k, name in _NAMES.items():
        f = C.c_void_p()
        r = _cu.cuModuleGetFunction(C.byref(f), _mod, name.encode())
        if r != 0:
            raise RuntimeError(f"cuModuleGetFunction({name}) failed: {r}")
        _fn[k] = f


def _launch(kernel, grid, block, args, stream):
    _load()
    holders = []
    for kind, v in args:
        holders.append(C.c_void_p(v) if kind == "p" else C.c_int(v))
    params = (C.c_void_p * len(holders))(*[C.cast(C.pointer(h), C.c_void_p) for h in holders])
    r = _cu.cuLaunchKernel(_fn[kernel], grid, 1, 1, block, 1, 1, 0,
                           C.c_void_p(stream or 0), params, None)
    if r != 0:
        raise RuntimeError(f"cuLaunchKernel({kernel}) failed: {r}")
    return 1


def eval_stencils(src, dst, length, src_stride, dst_stride, sizes, offsets, indices, weights,
                  start, end, stream=None):
    """CudaEvalStencils with device pointers (ints).  Returns the number of launches."""
    if length == 0 or src_stride == 0 or dst_stride == 0 or end <= start:
        return 0
    tab = [("p", sizes), ("p", offsets), ("p", indices), ("p", weights), ("i", start),
           ("i", end)]
    if length in (3, 4) and src_stride == length and dst_stride == length:
        grid = min(2048, (end - start + 255) // 256)
        return _launch("nv3" if length == 3 else "v4", grid, 256,
                       [("p", src), ("p", dst)] + tab, stream)
    return _launch("generic", 512, 32,
                   [("p", src), ("p", dst), ("i", length), ("i", src_stride),
                    ("i", dst_stride)] + tab, stream)


def eval_stencils_derivatives(src, outs, length, src_stride, strides, sizes, offsets, indices,
                              weights, start, end, stream=None):
    """CudaEvaluator::EvalStencils with derivatives: one CudaEvalStencils per output."""
    n = 0
    for dst, stride, w in zip(outs, strides, weights):
        if dst:
            n += eval_stencils(src, dst, length, src_stride, stride, sizes, offsets, indices, w,
                               start, end, stream)
    return n


def eval_patches(src, outs, length, src_stride, strides, n, coords, arrays, indices, params,
                 stream=None):
    """CudaEvalPatchesWithDerivatives: outs / strides for P, du, dv, duu, duv, dvv (0 = none)."""
    o = list(outs) + [0] * (6 - len(outs))
    st = list(strides) + [0] * (6 - len(strides))
    args = [("p", src)] + [("p", x) for x in o] + [("i", length), ("i", src_stride)] + \
        [("i", x) for x in st] + [("i", n), ("p", coords), ("p", arrays), ("p", indices),
                                   ("p", params)]
    return _launch("patches", 512, 32, args, stream)
