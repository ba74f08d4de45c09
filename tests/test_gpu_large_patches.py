"""EvalPatches at the size of the patch-evaluation benchmark, on the reference's own tables:
the 512 x 256 torus (seeded 5% triangles, 2% creases U[0, 4]) and the Loop icosphere
subdivided 6 times, both at adaptive isolation level 4 with Gregory-basis end caps, built by
Far::PatchTableFactory where the reference is available (tests/golden/make_golden.py large).

1 M uniform (ptex face, u, v) points per mesh: the device PatchMap must return Far's handles
bit for bit (the oracle's PatchMap, pinned to Far), and all six outputs pass the accuracy gate
(tests/gpu_util.py) against the oracle's CpuEvaluator and FP64 evaluations of the same coords.
"""
import os

import numpy as np
import pytest

import oracle
from gpu_util import bbox_diag, dev, gate, host, torch_cuda

LARGE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "large")
TABLES = ["torus512x256_adaptiveL4.npz", "icosphere6_loop_adaptiveL4.npz"]
POINTS = 1_000_000
THREADS = os.cpu_count() or 4


@pytest.mark.gpu
@pytest.mark.parametrize("name", TABLES)
def test_full_size_table_one_million_points_all_outputs(name):
    path = os.path.join(LARGE, name)
    if not os.path.exists(path):
        pytest.skip(f"{name} is written where the reference is available "
                    "(tests/golden/make_golden.py large)")
    torch = torch_cuda()
    from opensubdiv_gb300 import workloads
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300Evaluator as Ev
    from opensubdiv_gb300.evaluator import GB300PatchTable
    z = np.load(path)
    w = workloads.eval_patches_points(z, name[:-4], POINTS, seed=11)
    tri = bool(z["triangular"])
    t = GB300PatchTable.Create(w["arrays"], w["indices"], w["params"], tri)
    n = len(w["face"])
    coords = torch.zeros(n * 5, dtype=torch.int32, device="cuda")
    t.FindPatches(n, dev(w["face"]), dev(w["u"]), dev(w["v"]), coords)
    outs = [torch.zeros(n * 3, device="cuda") for _ in range(6)]
    d = BD(0, 3, 3)
    assert Ev.EvalPatchesTable(dev(w["src"]), d, outs[0], d, n, coords, t, du=outs[1],
                               duDesc=d, dv=outs[2], dvDesc=d, duu=outs[3], duuDesc=d,
                               duv=outs[4], duvDesc=d, dvv=outs[5], dvvDesc=d)
    Ev.Synchronize()
    c = np.ascontiguousarray(host(coords).reshape(n, 5))
    pm = oracle.PatchMap(w["arrays"], w["params"], tri)
    want = pm.find(w["face"], w["u"].astype(np.float64), w["v"].astype(np.float64))
    assert np.array_equal(c[:, :3], want)
    assert (c[:, 0] >= 0).all()  # every uniform query lands on a patch
    refs = [np.zeros(n * 3, np.float32) for _ in range(6)]
    f64s = [np.zeros(n * 3) for _ in range(6)]
    tab = (c, w["arrays"], w["indices"], w["params"])
    assert oracle.eval_patches(w["src"], (0, 3, 3), refs, [(0, 3, 3)] * 6, *tab, threads=THREADS)
    assert oracle.eval_patches(w["src"], (0, 3, 3), f64s, [(0, 3, 3)] * 6, *tab, threads=THREADS,
                               fp64=True)
    diag = bbox_diag(z["positions"])
    for k in range(6):
        gate(f"{name[:-4]} 1M points", k, host(outs[k]), refs[k], f64s[k], diag)
