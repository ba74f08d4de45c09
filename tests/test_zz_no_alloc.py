"""GB300EvalStencilsBatchedNoAlloc through the C ABI: a batched EvalStencils whose scratch is a
fixed device array inside the library (no allocation per call).

Two calls in a row, with different source values, must each match the existing
GB300EvalStencils entry point (one call per job) and the oracle (Osd::CpuEvaluator restated)
within the EvalStencils tolerance of 1e-5 x the cage's bounding-box diagonal, and leave the
library's device status word clear.  The file sorts last so that it also runs after every
other GPU test in the same process (and it passes alone).
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from gpu_util import bbox_diag, dev, host, max_err, torch_cuda

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REL_TOL = 1e-5
MAX_JOBS = 256


def _arr(ctype, values):
    return (ctype * len(values))(*values)


def _jobs(torch):
    """Jobs from the uniform-refinement fixtures: xyz at stride 3, and the 8-wide interleaved
    source at a descriptor offset (stride 8), several jobs per table."""
    jobs = []
    for name in ("cube8_uniform_L3", "torus32x16_uniform_L2", "icosphere2_uniform_L2",
                 "looptorus12x8_uniform_L2"):
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        tab = [dev(z[k]) for k in ("sizes", "offsets", "indices", "weights")]
        n = len(z["sizes"])
        diag = bbox_diag(z["positions"])
        src3 = z["src8"].reshape(-1, 8)[:, :3].copy().ravel()
        host_tab = [z[k] for k in ("sizes", "offsets", "indices", "weights")]
        jobs.append(dict(tab=tab, host_tab=host_tab, n=n, src=src3, length=3, sstride=3, soff=0,
                         dstride=3, doff=0, diag=diag))
        jobs.append(dict(tab=tab, host_tab=host_tab, n=n, src=z["src8"], length=5, sstride=8,
                         soff=2, dstride=7, doff=1, diag=diag))
    return jobs


def _call(lib, jobs, srcs, dsts, stream=None):
    n = len(jobs)
    P = C.c_void_p
    return lib.GB300EvalStencilsBatchedNoAlloc(
        n,
        _arr(P, [s.data_ptr() + 4 * j["soff"] for s, j in zip(srcs, jobs)]),
        _arr(P, [d.data_ptr() + 4 * j["doff"] for d, j in zip(dsts, jobs)]),
        _arr(C.c_int, [j["length"] for j in jobs]),
        _arr(C.c_int, [j["sstride"] for j in jobs]),
        _arr(C.c_int, [j["dstride"] for j in jobs]),
        _arr(C.c_int, [j["n"] for j in jobs]),
        _arr(P, [j["tab"][0].data_ptr() for j in jobs]),
        _arr(P, [j["tab"][1].data_ptr() for j in jobs]),
        _arr(P, [j["tab"][2].data_ptr() for j in jobs]),
        _arr(P, [j["tab"][3].data_ptr() for j in jobs]),
        stream)


@pytest.mark.gpu
def test_no_alloc_batch_matches_existing_entry_point_twice():
    torch = torch_cuda()
    from opensubdiv_gb300 import _lib
    lib = _lib.load()
    jobs = _jobs(torch)
    rng = np.random.default_rng(17)
    for call in range(2):
        # new source values for every call, so the second call must recompute everything
        hsrcs = [(j["src"] * (1.0 + 0.1 * call) + 0.01 * call).astype(np.float32)
                 for j in jobs]
        srcs = [dev(h) for h in hsrcs]
        dsts = [torch.full((j["n"] * j["dstride"],), float(rng.integers(2, 9)), device="cuda")
                for j in jobs]
        refs = [d.clone() for d in dsts]
        assert _call(lib, jobs, srcs, dsts) == 0, _lib.last_error()
        for j, s, r in zip(jobs, srcs, refs):
            assert lib.GB300EvalStencils(s.data_ptr() + 4 * j["soff"],
                                         r.data_ptr() + 4 * j["doff"], j["length"], j["sstride"],
                                         j["dstride"], j["tab"][0].data_ptr(),
                                         j["tab"][1].data_ptr(), j["tab"][2].data_ptr(),
                                         j["tab"][3].data_ptr(), 0, j["n"], None) == 0
        torch.cuda.synchronize()
        for k, (j, d, r) in enumerate(zip(jobs, dsts, refs)):
            g, e = host(d), host(r)
            tol = REL_TOL * j["diag"] * (1.0 + 0.1 * call)
            assert max_err(g, e) <= tol, f"call {call} job {k}"
            # the padding around each output row is left untouched
            gg = g.reshape(j["n"], j["dstride"])
            ee = e.reshape(j["n"], j["dstride"])
            keep = np.ones(j["dstride"], bool)
            keep[j["doff"]:j["doff"] + j["length"]] = False
            assert np.array_equal(gg[:, keep], ee[:, keep])
            # and the oracle on the same inputs
            o = np.zeros(j["n"] * j["length"], np.float32)
            assert oracle.eval_stencils(hsrcs[k], (j["soff"], j["length"], j["sstride"]), [o],
                                        [(0, j["length"], j["length"])], *j["host_tab"][:3],
                                        [j["host_tab"][3]], threads=4)
            got = gg[:, j["doff"]:j["doff"] + j["length"]].ravel()
            assert max_err(got, o) <= tol, f"call {call} job {k} vs oracle"
        # no bounded wait expired inside either call
        assert lib.GB300GetDeviceStatus() == 0, _lib.last_error()


@pytest.mark.gpu
def test_no_alloc_batch_rejects_more_jobs_than_its_scratch_holds():
    torch = torch_cuda()
    from opensubdiv_gb300 import _lib
    lib = _lib.load()
    jobs = _jobs(torch)[:1] * (MAX_JOBS + 1)
    srcs = [dev(jobs[0]["src"])] * len(jobs)
    dsts = [torch.zeros(jobs[0]["n"] * 3, device="cuda")] * len(jobs)
    assert _call(lib, jobs, srcs, dsts) == 1  # GB300_ERR_INVALID_ARGUMENT
    msg = _lib.last_error()
    assert "257 jobs" in msg and str(MAX_JOBS) in msg
    assert torch.count_nonzero(dsts[0]).item() == 0  # nothing was launched
