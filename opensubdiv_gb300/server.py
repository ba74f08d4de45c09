"""Python handle on the serving loop of libosd_gb300.so (GB300Server* in osd_gb300.h).

The server keeps topologies' stencil and patch tables resident under a device-memory budget
(LRU eviction), batches refine and limit-evaluation requests that are pending when a stream
frees up into one round, and overlaps rounds on several streams.  Requests carry host control
values and receive host results; use pinned host memory (``torch.empty(..., pin_memory=True)``)
so the copies stay asynchronous.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import GB300Error, check, last_error

REFINE, LIMIT = 0, 1


class ServerConfig(C.Structure):
    _fields_ = [("tableBudgetBytes", C.c_size_t), ("arenaBytes", C.c_size_t),
                ("streams", C.c_int), ("maxRequestsPerRound", C.c_int), ("plain", C.c_int),
                ("pinHostTables", C.c_int)]


class TopologyDesc(C.Structure):
    _fields_ = [("numControl", C.c_int), ("length", C.c_int), ("numStencils", C.c_int),
                ("nnz", C.c_int64), ("sizes", C.c_void_p), ("offsets", C.c_void_p),
                ("indices", C.c_void_p), ("weights", C.c_void_p),
                ("numPatchPoints", C.c_int), ("patchPointNnz", C.c_int64),
                ("ppSizes", C.c_void_p), ("ppOffsets", C.c_void_p), ("ppIndices", C.c_void_p),
                ("ppWeights", C.c_void_p), ("numPatchArrays", C.c_int),
                ("patchArrays", C.c_void_p), ("numPatchIndices", C.c_int64),
                ("patchIndices", C.c_void_p), ("numPatches", C.c_int),
                ("patchParams", C.c_void_p), ("triangular", C.c_int)]


class Request(C.Structure):
    _fields_ = [("topology", C.c_int), ("kind", C.c_int), ("controlValues", C.c_void_p),
                ("out", C.c_void_p), ("numPoints", C.c_int), ("faces", C.c_void_p),
                ("u", C.c_void_p), ("v", C.c_void_p)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "completed", "failed", "rounds",
                                          "uploads", "evictions", "bytesUploaded",
                                          "residentBytes", "peakResidentBytes", "launchNanos",
                                          "streamsBusyNanos", "memoryWaitNanos",
                                          "roundDeviceNanos", "h2dBytes", "d2hBytes",
                                          "hostPinnedBytes", "hostPinFailures")]


def _addr(a):
    """Host address of a numpy array or a (pinned) CPU torch tensor."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        if a.is_cuda:
            raise ValueError("server requests take host buffers")
        return a.data_ptr()
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("host arrays must be contiguous")
    return a.ctypes.data


def topology_desc(num_control, length, refine, limit=None):
    """A TopologyDesc over contiguous copies of the arrays; returns (desc, arrays to keep)."""
    r = {k: np.ascontiguousarray(refine[k], np.int32 if k != "weights" else np.float32)
         for k in ("sizes", "offsets", "indices", "weights")}
    d = TopologyDesc()
    d.numControl, d.length = int(num_control), int(length)
    d.numStencils, d.nnz = len(r["sizes"]), len(r["indices"])
    d.sizes, d.offsets, d.indices, d.weights = (_addr(r[k]) for k in
                                                ("sizes", "offsets", "indices", "weights"))
    keep = [r]
    if limit is not None:
        lm = {k: np.ascontiguousarray(limit[k], np.float32 if k == "pp_weights" else np.int32)
              for k in ("pp_sizes", "pp_offsets", "pp_indices", "pp_weights", "arrays",
                        "patch_indices", "params")}
        d.numPatchPoints, d.patchPointNnz = len(lm["pp_sizes"]), len(lm["pp_indices"])
        d.ppSizes, d.ppOffsets, d.ppIndices, d.ppWeights = (
            _addr(lm[k]) for k in ("pp_sizes", "pp_offsets", "pp_indices", "pp_weights"))
        d.numPatchArrays = lm["arrays"].shape[0]
        d.patchArrays = _addr(lm["arrays"])
        d.numPatchIndices = len(lm["patch_indices"])
        d.patchIndices = _addr(lm["patch_indices"])
        d.numPatches = lm["params"].shape[0]
        d.patchParams = _addr(lm["params"])
        d.triangular = int(bool(limit["triangular"]))
        keep.append(lm)
    return d, keep


def write_table_cache(path, num_control, length, refine, limit=None):
    """Write one topology's tables to a table-cache file (GB300TableCacheWrite)."""
    d, _keep = topology_desc(num_control, length, refine, limit)
    check(_lib.load().GB300TableCacheWrite(str(path).encode(), C.byref(d)))


def read_table_cache(path, verify=True):
    """Map a table-cache file and return copies of its arrays:
    (num_control, length, refine dict, limit dict or None)."""
    d = TopologyDesc()
    h = C.c_void_p()
    check(_lib.load().GB300TableCacheOpen(str(path).encode(), int(bool(verify)), C.byref(d),
                                          C.byref(h)))

    def arr(ptr, n, dtype, shape=None):
        if n == 0:
            return np.zeros(shape or (0,), dtype)
        ct = C.c_int32 if dtype == np.int32 else C.c_float
        a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), shape=(n,)).copy()
        return a.view(dtype).reshape(shape) if shape else a.view(dtype)

    try:
        refine = dict(sizes=arr(d.sizes, d.numStencils, np.int32),
                      offsets=arr(d.offsets, d.numStencils, np.int32),
                      indices=arr(d.indices, d.nnz, np.int32),
                      weights=arr(d.weights, d.nnz, np.float32))
        limit = None
        if d.numPatchArrays > 0:
            limit = dict(pp_sizes=arr(d.ppSizes, d.numPatchPoints, np.int32),
                         pp_offsets=arr(d.ppOffsets, d.numPatchPoints, np.int32),
                         pp_indices=arr(d.ppIndices, d.patchPointNnz, np.int32),
                         pp_weights=arr(d.ppWeights, d.patchPointNnz, np.float32),
                         arrays=arr(d.patchArrays, 6 * d.numPatchArrays, np.int32,
                                    (d.numPatchArrays, 6)),
                         patch_indices=arr(d.patchIndices, d.numPatchIndices, np.int32),
                         params=arr(d.patchParams, 3 * d.numPatches, np.int32,
                                    (d.numPatches, 3)),
                         triangular=bool(d.triangular))
        return d.numControl, d.length, refine, limit
    finally:
        _lib.load().GB300TableCacheClose(h)


class GB300Server:
    def __init__(self, table_budget_bytes, arena_bytes, streams=4, max_requests_per_round=64,
                 plain=False, pin_host_tables=False):
        cfg = ServerConfig(int(table_budget_bytes), int(arena_bytes), int(streams),
                           int(max_requests_per_round), int(bool(plain)),
                           int(bool(pin_host_tables)))
        self.handle = _lib.load().GB300ServerCreate(C.byref(cfg))
        if not self.handle:
            raise GB300Error(1, last_error())
        self._keep = {}  # host arrays the server reads until it is destroyed

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().GB300ServerDestroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    def add_topology(self, tid, num_control, length, refine, limit=None):
        """refine: dict(sizes, offsets, indices, weights) over the control vertices.
        limit: dict(pp_sizes, pp_offsets, pp_indices, pp_weights, arrays, patch_indices,
        params, triangular) or None."""
        d, keep = topology_desc(num_control, length, refine, limit)
        check(_lib.load().GB300ServerAddTopology(self.handle, int(tid), C.byref(d)))
        self._keep[int(tid)] = keep

    def add_topology_from_cache(self, tid, path):
        """Register a topology stored with write_table_cache (the server maps the file)."""
        check(_lib.load().GB300ServerAddTopologyFromCache(self.handle, int(tid),
                                                          str(path).encode()))

    @staticmethod
    def request(tid, kind, control_values, out, faces=None, u=None, v=None):
        q = Request()
        q.topology, q.kind = int(tid), int(kind)
        q.controlValues, q.out = _addr(control_values), _addr(out)
        if kind == LIMIT:
            q.numPoints = len(faces)
            q.faces, q.u, q.v = _addr(faces), _addr(u), _addr(v)
        return q

    def submit(self, req):
        t = C.c_uint64(0)
        check(_lib.load().GB300ServerSubmit(self.handle, C.byref(req), C.byref(t)))
        return t.value

    def wait(self, ticket):
        lat = C.c_double(0)
        check(_lib.load().GB300ServerWait(self.handle, C.c_uint64(ticket), C.byref(lat)))
        return lat.value

    def replay(self, reqs, arrivals):
        """Open-loop replay: request i submitted at arrivals[i] seconds; returns latencies."""
        n = len(reqs)
        arr = (Request * n)(*reqs)
        at = np.ascontiguousarray(arrivals, np.float64)
        lat = np.zeros(n, np.float64)
        check(_lib.load().GB300ServerReplay(self.handle, n, arr, at.ctypes.data,
                                            lat.ctypes.data))
        return lat

    def stats(self):
        s = ServerStats()
        check(_lib.load().GB300ServerGetStats(self.handle, C.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in ServerStats._fields_}
