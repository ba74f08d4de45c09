"""Python mirror of the Osd evaluator interface over libosd_gb300.so.

Names and argument meanings follow the reference's static evaluator API
(osd/cudaEvaluator.h:94-1262, osd/cpuEvaluator.h:39+) and its device-object wrappers
(CudaStencilTable osd/cudaEvaluator.h:52-92, CudaPatchTable osd/cudaPatchTable.h:51-110,
CudaVertexBuffer osd/cudaVertexBuffer.h:42-79):

* raw pointers (or CUDA tensors) exclude the BufferDescriptor offset; the evaluator adds it
  (cudaEvaluator.cpp:159-162);
* ``EvalStencils`` / ``EvalPatches`` return ``True`` on success and ``False`` on an invalid
  request (mismatched lengths, null table ...), like the reference's bool; the reason is in
  :func:`last_error`.  CUDA failures raise :class:`GB300Error`;
* work is queued on ``stream`` (a ``torch.cuda.Stream``, a raw ``cudaStream_t`` int or
  ``None`` for the legacy default stream); call :meth:`GB300Evaluator.Synchronize`.

Device memory is plain CUDA memory; torch tensors are accepted as a convenience.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import GB300Error, check, last_error  # noqa: F401

# Far::PatchDescriptor::Type values (far/patchDescriptor.h:48-63)
QUADS, TRIANGLES, LOOP, REGULAR, GREGORY_BASIS, GREGORY_TRIANGLE = 3, 4, 5, 6, 9, 10


@dataclass
class BufferDescriptor:
    """(offset, length, stride) of one primvar in an interleaved float buffer
    (osd/bufferDescriptor.h:61-103)."""

    offset: int = 0
    length: int = 0
    stride: int = 0

    def GetLocalOffset(self) -> int:
        return self.offset % self.stride if self.stride > 0 else 0

    def IsValid(self) -> bool:
        return self.length > 0 and self.length <= self.stride - self.GetLocalOffset()


def _ptr(x, offset_floats: int = 0):
    """Device address of x (+ offset in 4-byte elements) or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x + 4 * offset_floats
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise ValueError("GB300 evaluator buffers must live in device memory")
        return x.data_ptr() + 4 * offset_floats
    if hasattr(x, "BindCudaBuffer"):
        return x.BindCudaBuffer() + 4 * offset_floats
    raise TypeError(f"cannot take a device address of {type(x).__name__}")


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return s.cuda_stream  # torch.cuda.Stream


def _status_to_bool(status: int) -> bool:
    if status == 0:
        return True
    if status == 1:  # GB300_ERR_INVALID_ARGUMENT: the reference's `return false`
        return False
    raise GB300Error(status, last_error())


def _desc(d):
    return d if d is not None else BufferDescriptor()


class GB300Evaluator:
    """Static, stateless evaluator (drop-in beside CpuEvaluator / CudaEvaluator)."""

    @staticmethod
    def EvalStencils(src, srcDesc, dst, dstDesc, sizes, offsets, indices, weights,
                     start=0, end=None, du=None, duDesc=None, dv=None, dvDesc=None,
                     duWeights=None, dvWeights=None, duu=None, duuDesc=None, duv=None,
                     duvDesc=None, dvv=None, dvvDesc=None, duuWeights=None, duvWeights=None,
                     dvvWeights=None, stream=None) -> bool:
        """dst[i] = sum_j w_j src[idx_j] for stencils [start, end)
        (CudaEvaluator::EvalStencils, osd/cudaEvaluator.cpp:150-292).  The derivative forms
        run in the same single pass."""
        lib = _lib.load()
        if end is None:
            end = int(sizes.shape[0]) if hasattr(sizes, "shape") else 0
        outs = [(dst, dstDesc), (du, duDesc), (dv, dvDesc), (duu, duuDesc), (duv, duvDesc),
                (dvv, dvvDesc)]
        for o, d in outs:
            if o is not None and _desc(d).length != srcDesc.length:
                return False  # cpuEvaluator.cpp:46-47
        ws = [weights, duWeights, dvWeights, duuWeights, duvWeights, dvvWeights]
        if all(o is None for o, _ in outs[1:]):
            st = lib.GB300EvalStencils(_ptr(src, srcDesc.offset), _ptr(dst, dstDesc.offset),
                                       srcDesc.length, srcDesc.stride, dstDesc.stride,
                                       _ptr(sizes), _ptr(offsets), _ptr(indices), _ptr(weights),
                                       start, end, _stream(stream))
        else:
            ptrs = [_ptr(o, _desc(d).offset) if o is not None else None for o, d in outs]
            strides = [_desc(d).stride for _, d in outs]
            st = lib.GB300EvalStencilsWithDerivatives(
                _ptr(src, srcDesc.offset), *ptrs, srcDesc.length, srcDesc.stride, *strides,
                _ptr(sizes), _ptr(offsets), _ptr(indices),
                *[_ptr(w) if o is not None else None for w, (o, _) in zip(ws, outs)],
                start, end, _stream(stream))
        return _status_to_bool(st)

    @staticmethod
    def EvalStencilsTable(src, srcDesc, dst, dstDesc, table, du=None, duDesc=None, dv=None,
                          dvDesc=None, duu=None, duuDesc=None, duv=None, duvDesc=None,
                          dvv=None, dvvDesc=None, stream=None) -> bool:
        """Template form over a device table (osd/cudaEvaluator.h:125-142)."""
        outs = [(dst, dstDesc), (du, duDesc), (dv, dvDesc), (duu, duuDesc), (duv, duvDesc),
                (dvv, dvvDesc)]
        for o, d in outs:
            if o is not None and _desc(d).length != srcDesc.length:
                return False
        ptrs = [_ptr(o, _desc(d).offset) if o is not None else None for o, d in outs]
        strides = [_desc(d).stride for _, d in outs]
        st = _lib.load().GB300StencilTableEval(table.handle, _ptr(src, srcDesc.offset), *ptrs,
                                               srcDesc.length, srcDesc.stride, *strides,
                                               _stream(stream))
        return _status_to_bool(st)

    @staticmethod
    def EvalPatches(src, srcDesc, dst, dstDesc, numPatchCoords, patchCoords, patchArrays,
                    patchIndices, patchParams, du=None, duDesc=None, dv=None, dvDesc=None,
                    duu=None, duuDesc=None, duv=None, duvDesc=None, dvv=None, dvvDesc=None,
                    stream=None) -> bool:
        """Limit evaluation at patch coordinates (CudaEvaluator::EvalPatches,
        osd/cudaEvaluator.cpp:295-372)."""
        lib = _lib.load()
        outs = [(dst, dstDesc), (du, duDesc), (dv, dvDesc), (duu, duuDesc), (duv, duvDesc),
                (dvv, dvvDesc)]
        for o, d in outs:
            if o is not None and _desc(d).length != srcDesc.length:
                return False
        if all(o is None for o, _ in outs[1:]):
            st = lib.GB300EvalPatches(_ptr(src, srcDesc.offset), _ptr(dst, dstDesc.offset),
                                      srcDesc.length, srcDesc.stride, dstDesc.stride,
                                      numPatchCoords, _ptr(patchCoords), _ptr(patchArrays),
                                      _ptr(patchIndices), _ptr(patchParams), _stream(stream))
        else:
            ptrs = [_ptr(o, _desc(d).offset) if o is not None else None for o, d in outs]
            strides = [_desc(d).stride for _, d in outs]
            st = lib.GB300EvalPatchesWithDerivatives(
                _ptr(src, srcDesc.offset), *ptrs, srcDesc.length, srcDesc.stride, *strides,
                numPatchCoords, _ptr(patchCoords), _ptr(patchArrays), _ptr(patchIndices),
                _ptr(patchParams), _stream(stream))
        return _status_to_bool(st)

    @staticmethod
    def EvalPatchesTable(src, srcDesc, dst, dstDesc, numPatchCoords, patchCoords, table,
                         du=None, duDesc=None, dv=None, dvDesc=None, duu=None, duuDesc=None,
                         duv=None, duvDesc=None, dvv=None, dvvDesc=None, stream=None) -> bool:
        """Template form over a device patch table (osd/cudaEvaluator.h:502-525)."""
        outs = [(dst, dstDesc), (du, duDesc), (dv, dvDesc), (duu, duuDesc), (duv, duvDesc),
                (dvv, dvvDesc)]
        for o, d in outs:
            if o is not None and _desc(d).length != srcDesc.length:
                return False
        ptrs = [_ptr(o, _desc(d).offset) if o is not None else None for o, d in outs]
        strides = [_desc(d).stride for _, d in outs]
        st = _lib.load().GB300PatchTableEval(table.handle, _ptr(src, srcDesc.offset), *ptrs,
                                             srcDesc.length, srcDesc.stride, *strides,
                                             numPatchCoords, _ptr(patchCoords), _stream(stream))
        return _status_to_bool(st)

    @staticmethod
    def _eval_table_set(fn, lead, src, srcDesc, outs, numPatchCoords, patchCoords, stream):
        for o, d in outs:
            if o is not None and _desc(d).length != srcDesc.length:
                return False
        ptrs = [_ptr(o, _desc(d).offset) if o is not None else None for o, d in outs]
        strides = [_desc(d).stride for _, d in outs]
        st = fn(*lead, _ptr(src, srcDesc.offset), *ptrs, srcDesc.length, srcDesc.stride,
                *strides, numPatchCoords, _ptr(patchCoords), _stream(stream))
        return _status_to_bool(st)

    @staticmethod
    def EvalPatchesVarying(src, srcDesc, dst, dstDesc, numPatchCoords, patchCoords, table,
                           du=None, duDesc=None, dv=None, dvDesc=None, duu=None, duuDesc=None,
                           duv=None, duvDesc=None, dvv=None, dvvDesc=None, stream=None) -> bool:
        """Varying primvars at patch coords (osd/cudaEvaluator.h:859-1060)."""
        outs = [(dst, dstDesc), (du, duDesc), (dv, dvDesc), (duu, duuDesc), (duv, duvDesc),
                (dvv, dvvDesc)]
        return GB300Evaluator._eval_table_set(_lib.load().GB300PatchTableEvalVarying,
                                              (table.handle,), src, srcDesc, outs,
                                              numPatchCoords, patchCoords, stream)

    @staticmethod
    def EvalPatchesFaceVarying(src, srcDesc, dst, dstDesc, numPatchCoords, patchCoords, table,
                               fvarChannel=0, du=None, duDesc=None, dv=None, dvDesc=None,
                               duu=None, duuDesc=None, duv=None, duvDesc=None, dvv=None,
                               dvvDesc=None, stream=None) -> bool:
        """Face-varying primvars of channel fvarChannel at patch coords
        (osd/cudaEvaluator.h:1070-1255)."""
        outs = [(dst, dstDesc), (du, duDesc), (dv, dvDesc), (duu, duuDesc), (duv, duvDesc),
                (dvv, dvvDesc)]
        return GB300Evaluator._eval_table_set(_lib.load().GB300PatchTableEvalFaceVarying,
                                              (table.handle, int(fvarChannel)), src, srcDesc,
                                              outs, numPatchCoords, patchCoords, stream)

    @staticmethod
    def Synchronize(stream=None):
        check(_lib.load().GB300Synchronize(_stream(stream)))


class GB300StencilTable:
    """Device copy of a Far::StencilTable / LimitStencilTable (CudaStencilTable)."""

    def __init__(self, handle):
        self.handle = handle

    @classmethod
    def Create(cls, sizes, offsets, indices, weights, duWeights=None, dvWeights=None,
               duuWeights=None, duvWeights=None, dvvWeights=None, stream=None):
        """From host (numpy) arrays in Far layout; int32 sizes/offsets/indices, float32
        weights."""
        arrs = [np.ascontiguousarray(a, np.int32) for a in (sizes, offsets, indices)]
        ws = [np.ascontiguousarray(w, np.float32) if w is not None else None
              for w in (weights, duWeights, dvWeights, duuWeights, duvWeights, dvvWeights)]
        h = _lib.load().GB300StencilTableCreate(
            len(arrs[0]), len(arrs[2]), *[a.ctypes.data for a in arrs],
            *[w.ctypes.data if w is not None else None for w in ws], _stream(stream))
        if not h:
            raise GB300Error(3, last_error())
        return cls(h)

    def __del__(self):
        if getattr(self, "handle", None):
            _lib.load().GB300StencilTableDestroy(self.handle)
            self.handle = None

    def GetNumStencils(self):
        return _lib.load().GB300StencilTableGetNumStencils(self.handle)

    def _buf(self, k):
        return _lib.load().GB300StencilTableGetBuffer(self.handle, k)

    def GetNumIndices(self):
        return _lib.load().GB300StencilTableGetNumIndices(self.handle)

    def CopyToHost(self, stream=None):
        """The table's device arrays as numpy arrays (Far names: sizes, offsets, indices,
        weights and, where present, du_weights ... dvv_weights)."""
        n, nnz = self.GetNumStencils(), self.GetNumIndices()
        names = ("sizes", "offsets", "indices", "weights", "du_weights", "dv_weights",
                 "duu_weights", "duv_weights", "dvv_weights")
        out = {}
        for k, name in enumerate(names):
            if not self._buf(k):
                continue
            a = np.zeros(n if k < 2 else nnz, np.int32 if k < 3 else np.float32)
            check(_lib.load().GB300StencilTableCopyBuffer(self.handle, k, a.ctypes.data,
                                                          _stream(stream)))
            out[name] = a
        return out

    @classmethod
    def ComposeRows(cls, base, offsets, sources, weights, appendBase=False, sortEntries=True,
                    stream=None):
        """Stencils composed over the rows of a device table `base` (a GB300StencilTable
        whose entries are in Far's order, e.g. from GB300StencilTableFactory.Create with
        sortEntries=False): row i merges weights[c][k] * w over the entries (index, w) of base
        stencil sources[k] (StencilBuilder::Index::AddWithWeight with a StencilReal source,
        far/stencilBuilder.cpp:520-598).  weights: list of 1, 3 or 6 host float32 arrays."""
        off = np.ascontiguousarray(offsets, np.int64)
        src = np.ascontiguousarray(sources, np.int32)
        ws = [np.ascontiguousarray(w, np.float32) for w in weights]
        wp = (C.c_void_p * len(ws))(*[w.ctypes.data for w in ws])
        L = _lib.load()
        h = L.GB300StencilTableComposeRows(
            base.GetNumStencils(), base.GetNumIndices(), base.GetSizesBuffer(),
            base.GetOffsetsBuffer(), base.GetIndicesBuffer(), base.GetWeightsBuffer(),
            len(off) - 1, len(src), off.ctypes.data, src.ctypes.data if len(src) else None,
            len(ws), wp, int(bool(appendBase)), int(bool(sortEntries)), _stream(stream))
        if not h:
            raise GB300Error(1, last_error())
        return cls(h)

    @classmethod
    def FromPatchCoords(cls, table, patch_coords, base, num_points=None, channels=3,
                        sortEntries=True, stream=None):
        """Bfr::Surface::EvaluateStencil at every point (GB300TessellationStencils): one limit
        stencil per PatchCoord of the GB300PatchTable `table` (a CUDA tensor of [n, 5] int32,
        e.g. from MeshTessellation.Generate or Share), over the control vertices, composed
        over `base` -- a GB300StencilTable holding one stencil per point the patch indices
        name (identity rows for the control vertices, then the refined and local points).
        channels: 1 (P), 3 (P, Du, Dv) or 6 (with the second derivatives)."""
        n = int(patch_coords.shape[0]) if num_points is None else int(num_points)
        h = _lib.load().GB300TessellationStencils(
            table.handle, n, _ptr(patch_coords), base.GetNumStencils(), base.GetNumIndices(),
            base.GetSizesBuffer(), base.GetOffsetsBuffer(), base.GetIndicesBuffer(),
            base.GetWeightsBuffer(), int(channels), int(bool(sortEntries)), _stream(stream))
        if not h:
            raise GB300Error(1, last_error())
        return cls(h)

    def GetSizesBuffer(self): return self._buf(0)
    def GetOffsetsBuffer(self): return self._buf(1)
    def GetIndicesBuffer(self): return self._buf(2)
    def GetWeightsBuffer(self): return self._buf(3)
    def GetDuWeightsBuffer(self): return self._buf(4)
    def GetDvWeightsBuffer(self): return self._buf(5)
    def GetDuuWeightsBuffer(self): return self._buf(6)
    def GetDuvWeightsBuffer(self): return self._buf(7)
    def GetDvvWeightsBuffer(self): return self._buf(8)


class _StencilMasks(C.Structure):
    _fields_ = [("numRows", C.c_int), ("nnz", C.c_int64), ("offsets", C.c_void_p),
                ("sources", C.c_void_p), ("weights", C.c_void_p)]


class GB300StencilTableFactory:
    """Far::StencilTableFactory::Create (factorized) with the merging on the GPU, from the
    per-level masks Far::PrimvarRefiner produces (as recorded by GB300MaskRecorder in
    include/opensubdiv_gb300/far/gb300StencilTableFactory.h)."""

    @staticmethod
    def Create(numControl, levels, generateIntermediateLevels=True, generateControlVerts=False,
               sortEntries=True, stream=None):
        """levels: per refinement level a dict of host arrays offsets (int64, rows + 1),
        sources (int32, global vertex indices) and weights (float32).  sortEntries=False keeps
        each stencil's entries in Far's order (the table then equals Far's bit for bit)."""
        keep = []
        views = (_StencilMasks * max(1, len(levels)))()
        for i, d in enumerate(levels):
            off = np.ascontiguousarray(d["offsets"], np.int64)
            src = np.ascontiguousarray(d["sources"], np.int32)
            w = np.ascontiguousarray(d["weights"], np.float32)
            keep += [off, src, w]
            views[i] = _StencilMasks(len(off) - 1, len(src), off.ctypes.data,
                                     src.ctypes.data if len(src) else None,
                                     w.ctypes.data if len(w) else None)
        h = _lib.load().GB300StencilTableFactoryCreate(
            int(numControl), len(levels), C.cast(views, C.c_void_p),
            int(bool(generateIntermediateLevels)), int(bool(generateControlVerts)),
            int(bool(sortEntries)), _stream(stream))
        if not h:
            raise GB300Error(1, last_error())
        return GB300StencilTable(h)


class GB300StencilBatch:
    """Many meshes' EvalStencils in one persistent launch (no counterpart in the reference;
    the per-mesh equivalent is one EvalStencilsTable call per job).

    ``jobs`` is a sequence of ``(table, src, srcDesc, dst, dstDesc)``: a
    :class:`GB300StencilTable` and device buffers with their descriptors, as for
    :meth:`GB300Evaluator.EvalStencilsTable`.  Tables and buffers must outlive the batch."""

    def __init__(self, jobs, stream=None):
        import ctypes as C
        n = len(jobs)
        tabs = (C.c_void_p * n)()
        srcs = (C.c_void_p * n)()
        dsts = (C.c_void_p * n)()
        lens, sst, dst_ = (C.c_int * n)(), (C.c_int * n)(), (C.c_int * n)()
        for i, (table, src, sd, dst, dd) in enumerate(jobs):
            sd, dd = _desc(sd), _desc(dd)
            if sd.length != dd.length or not sd.IsValid() or not dd.IsValid():
                raise ValueError(f"job {i}: mismatched or invalid buffer descriptors")
            tabs[i] = table.handle
            srcs[i] = _ptr(src, sd.offset)
            dsts[i] = _ptr(dst, dd.offset)
            lens[i], sst[i], dst_[i] = sd.length, sd.stride, dd.stride
        self._keep = [j[0] for j in jobs]  # tables stay alive while the batch exists
        self.handle = _lib.load().GB300StencilBatchCreate(n, tabs, srcs, dsts, lens, sst, dst_,
                                                          _stream(stream))
        if not self.handle:
            raise GB300Error(1, last_error())

    def __del__(self):
        if getattr(self, "handle", None):
            _lib.load().GB300StencilBatchDestroy(self.handle)
            self.handle = None

    def Eval(self, stream=None):
        check(_lib.load().GB300StencilBatchEval(self.handle, _stream(stream)))

    def EvalGraph(self, stream=None):
        check(_lib.load().GB300StencilBatchEvalGraph(self.handle, _stream(stream)))

    def Tune(self, iterations=3, stream=None):
        check(_lib.load().GB300StencilBatchTune(self.handle, iterations, _stream(stream)))

    def GetConfig(self):
        import ctypes as C
        v = [C.c_int(0) for _ in range(5)]
        check(_lib.load().GB300StencilBatchGetConfig(self.handle, *[C.byref(x) for x in v]))
        return dict(tile_stencils=v[0].value, ctas_per_sm=v[1].value,
                    warp_threshold=v[2].value, num_tiles=v[3].value,
                    dynamic_claims=v[4].value)

    def GetDeviceStatus(self):
        import ctypes as C
        s = C.c_int(0)
        check(_lib.load().GB300StencilBatchGetDeviceStatus(self.handle, C.byref(s)))
        return s.value


class GB300PatchTable:
    """Device copy of a flattened Far::PatchTable plus its device PatchMap (CudaPatchTable)."""

    def __init__(self, handle):
        self.handle = handle

    @classmethod
    def Create(cls, arrays, indices, params, triangular=False, stream=None):
        """From host arrays in Osd::CpuPatchTable layout: int32 [nArrays, 6] patch arrays,
        int32 index buffer, int32 [nPatches, 3] params (field0, field1, sharpness bits)."""
        a = np.ascontiguousarray(arrays, np.int32)
        i = np.ascontiguousarray(indices, np.int32)
        p = np.ascontiguousarray(params, np.int32)
        h = _lib.load().GB300PatchTableCreate(len(a), a.ctypes.data, len(i), i.ctypes.data,
                                              len(p), p.ctypes.data, int(bool(triangular)),
                                              _stream(stream))
        if not h:
            raise GB300Error(1, last_error())
        return cls(h)

    def __del__(self):
        if getattr(self, "handle", None):
            _lib.load().GB300PatchTableDestroy(self.handle)
            self.handle = None

    def GetPatchArrayBuffer(self): return _lib.load().GB300PatchTableGetBuffer(self.handle, 0)
    def GetPatchIndexBuffer(self): return _lib.load().GB300PatchTableGetBuffer(self.handle, 1)
    def GetPatchParamBuffer(self): return _lib.load().GB300PatchTableGetBuffer(self.handle, 2)

    def SetVarying(self, arrays, indices, stream=None):
        """Varying patch arrays / indices (CpuPatchTable's varying tables), evaluated with the
        vertex patch params."""
        a = np.ascontiguousarray(arrays, np.int32)
        i = np.ascontiguousarray(indices, np.int32)
        check(_lib.load().GB300PatchTableSetVarying(self.handle, len(a), a.ctypes.data, len(i),
                                                    i.ctypes.data, _stream(stream)))

    def AddFVarChannel(self, arrays, indices, params, stream=None):
        """Face-varying channel tables; returns the channel index."""
        import ctypes as C
        a = np.ascontiguousarray(arrays, np.int32)
        i = np.ascontiguousarray(indices, np.int32)
        p = np.ascontiguousarray(params, np.int32)
        ch = C.c_int(-1)
        check(_lib.load().GB300PatchTableAddFVarChannel(self.handle, len(a), a.ctypes.data,
                                                        len(i), i.ctypes.data, len(p),
                                                        p.ctypes.data, C.byref(ch),
                                                        _stream(stream)))
        return ch.value

    def GetNumFVarChannels(self):
        return _lib.load().GB300PatchTableGetNumFVarChannels(self.handle)

    def GetVaryingPatchArrayBuffer(self):
        return _lib.load().GB300PatchTableGetVaryingBuffer(self.handle, 0)

    def GetVaryingPatchIndexBuffer(self):
        return _lib.load().GB300PatchTableGetVaryingBuffer(self.handle, 1)

    def GetFVarPatchArrayBuffer(self, channel=0):
        return _lib.load().GB300PatchTableGetFVarBuffer(self.handle, channel, 0)

    def GetFVarPatchIndexBuffer(self, channel=0):
        return _lib.load().GB300PatchTableGetFVarBuffer(self.handle, channel, 1)

    def GetFVarPatchParamBuffer(self, channel=0):
        return _lib.load().GB300PatchTableGetFVarBuffer(self.handle, channel, 2)

    def TessFactors(self, options, outer, inner, outer_lo=None, outer_hi=None, src=None,
                    src_stride=3, stream=None):
        """Draw-time tessellation factors of every patch (GB300PatchTableTessFactors):
        outer [numPatches, 4], inner [numPatches, 2] and optionally the Lo / Hi outer halves
        [numPatches, 4]; `options` is a PatchTessOptions."""
        import ctypes as C
        check(_lib.load().GB300PatchTableTessFactors(
            self.handle, _ptr(src), int(src_stride), C.byref(options), _ptr(outer), _ptr(inner),
            _ptr(outer_lo), _ptr(outer_hi), _stream(stream)))

    def FindPatches(self, n, faces, u, v, coords_out, stream=None):
        """Device PatchMap lookup: writes n OsdPatchCoord records to coords_out."""
        check(_lib.load().GB300PatchTableFindPatches(self.handle, n, _ptr(faces), _ptr(u),
                                                     _ptr(v), _ptr(coords_out), _stream(stream)))


class PatchTessOptions(C.Structure):
    """The patch shaders' tess-control settings (OsdTessLevel, the device maximum level,
    screen-space tessellation, spacing 0 equal / 1 fractional even / 2 fractional odd, and the
    model-view and projection matrices as 4x4 arrays in the usual row-major math layout; they
    are stored column-major like a GLSL mat4)."""

    _fields_ = [("tessLevel", C.c_float), ("maxTessLevel", C.c_float),
                ("screenSpace", C.c_int), ("spacing", C.c_int),
                ("modelView", C.c_float * 16), ("projection", C.c_float * 16)]

    def __init__(self, tess_level=1.0, max_tess_level=64.0, screen_space=False, spacing=0,
                 model_view=None, projection=None):
        super().__init__()
        self.tessLevel = float(tess_level)
        self.maxTessLevel = float(max_tess_level)
        self.screenSpace = int(bool(screen_space))
        self.spacing = int(spacing)
        mv = np.asarray(model_view if model_view is not None else np.eye(4), np.float32)
        pr = np.asarray(projection if projection is not None else np.eye(4), np.float32)
        self.modelView[:] = mv.T.ravel().tolist()
        self.projection[:] = pr.T.ravel().tolist()


def PatchTessParameterization(n, domain, patch_index, outer_lo, outer_hi, uv, spacing=0,
                              triangular=False, stream=None):
    """OsdGetTessParameterization[Triangle] on the device (GB300PatchTessParameterization):
    n domain points (u, v, w) of patches patch_index -> patch (u, v) in uv."""
    check(_lib.load().GB300PatchTessParameterization(
        int(n), _ptr(domain), _ptr(patch_index), _ptr(outer_lo), _ptr(outer_hi), int(spacing),
        int(bool(triangular)), _ptr(uv), _stream(stream)))


class GB300VertexBuffer:
    """Owning device float buffer of numVertices x numElements (CudaVertexBuffer)."""

    def __init__(self, handle):
        self.handle = handle

    @classmethod
    def Create(cls, numElements, numVertices, deviceContext=None):
        h = _lib.load().GB300VertexBufferCreate(numElements, numVertices)
        if not h:
            raise GB300Error(3, last_error())
        return cls(h)

    def __del__(self):
        if getattr(self, "handle", None):
            _lib.load().GB300VertexBufferDestroy(self.handle)
            self.handle = None

    def UpdateData(self, src, startVertex, numVertices, stream=None):
        src = np.ascontiguousarray(src, np.float32)
        check(_lib.load().GB300VertexBufferUpdateData(self.handle, src.ctypes.data, startVertex,
                                                      numVertices, _stream(stream)))

    def BindCudaBuffer(self) -> int:
        return _lib.load().GB300VertexBufferBindCudaBuffer(self.handle)

    def GetNumElements(self): return _lib.load().GB300VertexBufferGetNumElements(self.handle)
    def GetNumVertices(self): return _lib.load().GB300VertexBufferGetNumVertices(self.handle)
