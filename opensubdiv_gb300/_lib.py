"""Loader for libosd_gb300.so, the C ABI declared in include/osd_gb300.h.

The evaluator has no CPU fallback: if the shared library is missing or cannot be loaded,
every call raises.  ``load(build=True)`` compiles it first with nvcc (sm_103a).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

LIB_PATH = _build.LIB

_lib = None
_lock = threading.Lock()

vp, i32, i64, u64 = C.c_void_p, C.c_int, C.c_int64, C.c_uint64

_PROTOS = {
    "GB300GetLastErrorString": (C.c_char_p, []),
    "GB300GetVersion": (i32, []),
    "GB300Synchronize": (i32, [vp]),
    "GB300GetLaunchCount": (u64, []),
    "GB300GetDeviceStatus": (i32, []),
    "GB300MeasureFp32Rate": (i32, [C.POINTER(C.c_double), vp]),
    "GB300EvalStencils": (i32, [vp, vp, i32, i32, i32, vp, vp, vp, vp, i32, i32, vp]),
    "GB300EvalStencilsWithDerivatives": (
        i32, [vp] * 7 + [i32] * 8 + [vp] * 3 + [vp] * 6 + [i32, i32, vp]),
    "GB300EvalPatches": (i32, [vp, vp, i32, i32, i32, i32, vp, vp, vp, vp, vp]),
    "GB300EvalPatchesWithDerivatives": (i32, [vp] * 7 + [i32] * 8 + [i32] + [vp] * 4 + [vp]),
    "GB300StencilTableCreate": (vp, [i32, i64] + [vp] * 9 + [vp]),
    "GB300StencilTableDestroy": (None, [vp]),
    "GB300StencilTableGetNumStencils": (i32, [vp]),
    "GB300StencilTableGetNumIndices": (i64, [vp]),
    "GB300StencilTableGetBuffer": (vp, [vp, i32]),
    "GB300StencilTableEval": (i32, [vp, vp] + [vp] * 6 + [i32] * 8 + [vp]),
    "GB300StencilTableCopyBuffer": (i32, [vp, i32, vp, vp]),
    "GB300StencilTableFactoryCreate": (vp, [i32, i32, vp, i32, i32, i32, vp]),
    "GB300StencilTableComposeRows": (vp, [i32, i64, vp, vp, vp, vp, i32, i64, vp, vp, i32, vp,
                                          i32, i32, vp]),
    "GB300PatchTableCreate": (vp, [i32, vp, i64, vp, i32, vp, i32, vp]),
    "GB300PatchTableDestroy": (None, [vp]),
    "GB300PatchTableGetBuffer": (vp, [vp, i32]),
    "GB300PatchTableGetNumArrays": (i32, [vp]),
    "GB300PatchTableGetNumPatches": (i32, [vp]),
    "GB300PatchTableFindPatches": (i32, [vp, i32, vp, vp, vp, vp, vp]),
    "GB300PatchTableEval": (i32, [vp, vp] + [vp] * 6 + [i32] * 8 + [i32, vp, vp]),
    "GB300PatchTableSetVarying": (i32, [vp, i32, vp, i64, vp, vp]),
    "GB300PatchTableAddFVarChannel": (i32, [vp, i32, vp, i64, vp, i32, vp, vp, vp]),
    "GB300PatchTableGetNumFVarChannels": (i32, [vp]),
    "GB300PatchTableGetVaryingBuffer": (vp, [vp, i32]),
    "GB300PatchTableGetFVarBuffer": (vp, [vp, i32, i32]),
    "GB300PatchTableEvalVarying": (i32, [vp, vp] + [vp] * 6 + [i32] * 8 + [i32, vp, vp]),
    "GB300PatchTableEvalFaceVarying": (i32, [vp, i32, vp] + [vp] * 6 + [i32] * 8 + [i32, vp, vp]),
    "GB300TessellationCount": (i32, [i32, i32, vp, vp, vp, i32, vp, vp, vp, vp, vp, vp]),
    "GB300TessellationGenerate": (i32, [i32, i32, vp, vp, vp, i32, vp, vp, vp, vp, vp, vp, i32,
                                        vp, vp, vp]),
    "GB300TessellationEvaluate": (i32, [vp, vp] + [vp] * 6 + [i32] * 8 + [i32, vp, vp]),
    "GB300TessellationEdgeRates": (i32, [i32, vp, vp, i64, vp, i32, i32, i32, C.c_float, i32,
                                         vp, vp, vp]),
    "GB300TessellationStencils": (vp, [vp, i32, vp, i32, i64, vp, vp, vp, vp, i32, i32, vp]),
    "GB300TessellationShare": (i32, [i32, i32, vp, vp, vp, i32, vp, vp, vp, vp, vp, i64, i32,
                                     i32, vp, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "GB300PatchTableTessFactors": (i32, [vp, vp, i32, vp, vp, vp, vp, vp, vp]),
    "GB300PatchTessParameterization": (i32, [i32, vp, vp, vp, vp, i32, i32, vp, vp]),
    "GB300VertexBufferCreate": (vp, [i32, i32]),
    "GB300VertexBufferDestroy": (None, [vp]),
    "GB300VertexBufferUpdateData": (i32, [vp, vp, i32, i32, vp]),
    "GB300VertexBufferBindCudaBuffer": (vp, [vp]),
    "GB300VertexBufferGetNumElements": (i32, [vp]),
    "GB300VertexBufferGetNumVertices": (i32, [vp]),
    "GB300StencilBatchCreate": (vp, [i32, vp, vp, vp, vp, vp, vp, vp]),
    "GB300StencilBatchDestroy": (None, [vp]),
    "GB300StencilBatchEval": (i32, [vp, vp]),
    "GB300StencilBatchEvalGraph": (i32, [vp, vp]),
    "GB300StencilBatchTune": (i32, [vp, i32, vp]),
    "GB300StencilBatchGetConfig": (i32, [vp, vp, vp, vp, vp, vp]),
    "GB300StencilBatchGetDeviceStatus": (i32, [vp, vp]),
    "GB300EvalStencilsBatchedNoAlloc": (i32, [i32] + [vp] * 11),
    "GB300ServerCreate": (vp, [vp]),
    "GB300ServerDestroy": (None, [vp]),
    "GB300ServerAddTopology": (i32, [vp, i32, vp]),
    "GB300ServerSubmit": (i32, [vp, vp, vp]),
    "GB300ServerWait": (i32, [vp, u64, vp]),
    "GB300ServerReplay": (i32, [vp, i32, vp, vp, vp]),
    "GB300ServerGetStats": (i32, [vp, vp]),
    "GB300ServerAddTopologyFromCache": (i32, [vp, i32, C.c_char_p]),
    "GB300TableCacheWrite": (i32, [C.c_char_p, vp]),
    "GB300TableCacheOpen": (i32, [C.c_char_p, i32, vp, vp]),
    "GB300TableCacheClose": (None, [vp]),
}


class GB300Error(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[status {code}] {message}")
        self.code = code


def load(build: bool = False):
    """Returns the ctypes handle, compiling the library first when asked (or when it has
    never been built here)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build or not os.path.exists(LIB_PATH):
            _build.build()
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def exported_symbols():
    return list(_PROTOS)


def last_error() -> str:
    msg = load().GB300GetLastErrorString()
    return msg.decode() if msg else ""


def check(status: int):
    if status != 0:
        raise GB300Error(status, last_error())
    return status


def launch_count() -> int:
    return int(load().GB300GetLaunchCount())
