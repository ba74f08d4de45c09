"""Parity on the plain-method workload itself, at full size: the 512 x 256 torus (R = 1,
r = 0.3; seeded 5% triangle splits, 2% creases U[0, 4]) refined uniformly to Catmull-Clark
level 3 (8,598,400 stencils, 112 M entries) over 8 interleaved float32 primvars, plus limit
stencils with du/dv weights at 1 M seeded (ptex face, u, v) locations.  Every output of the
device-table EvalStencils (the sliced kernel the throughput figures time) is compared with the
oracle (Osd::CpuEvaluator restated, run on all host threads) at 1e-5 x the cage's
bounding-box diagonal, with the float tables applied in double reported beside it."""
import os

import numpy as np
import pytest

import oracle
from gpu_util import bbox_diag, dev, gate, host, torch_cuda

THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module")
def headline():
    from opensubdiv_gb300 import workloads
    return workloads.refine_and_limit_torus()


@pytest.mark.gpu
def test_headline_refine_all_primvars(headline):
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300Evaluator as Ev
    from opensubdiv_gb300.evaluator import GB300StencilTable
    w = headline
    r, L, src = w["refine"], w["length"], w["src"]
    n = len(r["sizes"])
    assert n == 8_598_400 and L == 8
    t = GB300StencilTable.Create(r["sizes"], r["offsets"], r["indices"], r["weights"])
    d = BD(0, L, L)
    out = torch.zeros(n * L, device="cuda")
    assert Ev.EvalStencilsTable(dev(src), d, out, d, t)
    Ev.Synchronize()
    ref = np.zeros(n * L, np.float32)
    f64 = np.zeros(n * L)
    for o, fp in ((ref, False), (f64, True)):
        assert oracle.eval_stencils(src, (0, L, L), [o], [(0, L, L)], r["sizes"], r["offsets"],
                                    r["indices"], [r["weights"]], threads=THREADS, fp64=fp)
    gate("torus512x256 L3 refine, 8 primvars", 0, host(out), ref, f64,
         bbox_diag(w["cage"].positions))


@pytest.mark.gpu
def test_headline_limit_p_du_dv(headline):
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300Evaluator as Ev
    from opensubdiv_gb300.evaluator import GB300StencilTable
    w = headline
    lim, L, src = w["limit"], w["length"], w["src"]
    m = len(lim["sizes"])
    assert m == 1_000_000
    ws = [lim["weights"], lim["du_weights"], lim["dv_weights"]]
    t = GB300StencilTable.Create(lim["sizes"], lim["offsets"], lim["indices"], *ws)
    d = BD(0, L, L)
    outs = [torch.zeros(m * L, device="cuda") for _ in range(3)]
    assert Ev.EvalStencilsTable(dev(src), d, outs[0], d, t, du=outs[1], duDesc=d, dv=outs[2],
                                dvDesc=d)
    Ev.Synchronize()
    refs = [np.zeros(m * L, np.float32) for _ in range(3)]
    f64s = [np.zeros(m * L) for _ in range(3)]
    for o, fp in ((refs, False), (f64s, True)):
        assert oracle.eval_stencils(src, (0, L, L), o, [(0, L, L)] * 3, lim["sizes"],
                                    lim["offsets"], lim["indices"], ws, threads=THREADS, fp64=fp)
    diag = bbox_diag(w["cage"].positions)
    for k in range(3):
        gate("torus512x256 limit 1M, 8 primvars", k, host(outs[k]), refs[k], f64s[k], diag)
