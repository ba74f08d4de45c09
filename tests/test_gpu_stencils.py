"""EvalStencils on the GB300 through the C ABI, checked against the oracle.

The oracle reproduces Osd::CpuEvaluator bit for bit (tests/test_oracle_golden.py), so
"oracle" below means "the reference's CPU evaluator on the same inputs".  Tolerance, per the
accuracy contract: max |gpu - cpu| <= 1e-5 x the cage's bounding-box diagonal (the GPU
accumulates with fused multiply-adds, so results are not bitwise equal); the error of both
against the FP64 oracle (same tables, double accumulation) is reported alongside.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from gpu_util import bbox_diag, dev, gate, host, max_err, torch_cuda

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "*_uniform_L*.npz")))
REL_TOL = 1e-5


def _ev():
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300Evaluator as Ev
    return Ev, BD


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_eval_stencils_matches_cpu(path):
    torch = torch_cuda()
    Ev, BD = _ev()
    z = np.load(path)
    n = len(z["sizes"])
    tol = REL_TOL * bbox_diag(z["positions"])
    tbl = [dev(z[k]) for k in ("sizes", "offsets", "indices", "weights")]
    # xyz, stride 3
    src = dev(z["positions"].ravel())
    out = torch.zeros(n * 3, device="cuda")
    assert Ev.EvalStencils(src, BD(0, 3, 3), out, BD(0, 3, 3), *tbl, 0, n)
    Ev.Synchronize()
    assert max_err(host(out), z["out3"]) <= tol
    # 8 interleaved primvars
    src8 = dev(z["src8"])
    out8 = torch.zeros(n * 8, device="cuda")
    assert Ev.EvalStencils(src8, BD(0, 8, 8), out8, BD(0, 8, 8), *tbl, 0, n)
    Ev.Synchronize()
    assert max_err(host(out8), z["out8"]) <= tol
    # offsets and strides: source (2, 3, 7), destination (1, 3, 5); untouched lanes stay 0
    src7 = dev(z["src7"])
    out5 = torch.zeros(n * 5 + 5, device="cuda")
    assert Ev.EvalStencils(src7, BD(2, 3, 7), out5, BD(1, 3, 5), *tbl, 0, n)
    Ev.Synchronize()
    o5 = host(out5)
    assert max_err(o5, z["out_strided"]) <= tol
    assert np.all(o5.reshape(-1, 5)[:-1, [0, 4]] == 0)
    # in place, one buffer, destination after the control points (osd/mesh.h:501-540)
    nc = len(z["positions"])
    buf = torch.zeros((nc + n) * 3, device="cuda")
    buf[: nc * 3] = src
    assert Ev.EvalStencils(buf, BD(0, 3, 3), buf, BD(nc * 3, 3, 3), *tbl, 0, n)
    Ev.Synchronize()
    assert max_err(host(buf), z["out_inplace"]) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_eval_stencils_device_table_and_fp64(path):
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import GB300StencilTable
    Ev, BD = _ev()
    z = np.load(path)
    n = len(z["sizes"])
    diag = bbox_diag(z["positions"])
    table = GB300StencilTable.Create(z["sizes"], z["offsets"], z["indices"], z["weights"])
    assert table.GetNumStencils() == n
    src = dev(z["positions"].ravel())
    out = torch.zeros(n * 3, device="cuda")
    assert Ev.EvalStencilsTable(src, BD(0, 3, 3), out, BD(0, 3, 3), table)
    Ev.Synchronize()
    g = host(out)
    assert max_err(g, z["out3"]) <= REL_TOL * diag
    o64 = np.zeros(n * 3)
    oracle.eval_stencils(z["positions"].ravel(), (0, 3, 3), [o64], [(0, 3, 3)], z["sizes"],
                         z["offsets"], z["indices"], [z["weights"]], fp64=True)
    e_gpu, e_cpu = max_err(g, o64), max_err(z["out3"], o64)
    print(f"{os.path.basename(path)}: |gpu-fp64|={e_gpu:.2e} |cpu-fp64|={e_cpu:.2e} "
          f"(diag {diag:.3f})")
    assert e_gpu <= REL_TOL * diag


@pytest.mark.gpu
@pytest.mark.parametrize("path", [p for p in FIXTURES if "limit_sizes" in np.load(p)],
                         ids=os.path.basename)
@pytest.mark.parametrize("nout", [1, 2, 3, 4, 5, 6])
def test_limit_stencils_fused_derivatives(path, nout):
    torch = torch_cuda()
    Ev, BD = _ev()
    z = np.load(path)
    m = len(z["limit_sizes"])
    diag = bbox_diag(z["positions"])
    names = ("weights", "du_weights", "dv_weights", "duu_weights", "duv_weights", "dvv_weights")
    ws = [dev(z["limit_" + k]) for k in names]
    tbl = [dev(z["limit_" + k]) for k in ("sizes", "offsets", "indices")]
    src = dev(z["positions"].ravel())
    outs = [torch.zeros(m * 3, device="cuda") for _ in range(6)]
    kw = {}
    keys = ("du", "dv", "duu", "duv", "dvv")
    for k in range(1, nout):
        kw[keys[k - 1]] = outs[k]
        kw[keys[k - 1] + "Desc"] = BD(0, 3, 3)
        kw[keys[k - 1] + "Weights"] = ws[k]
    assert Ev.EvalStencils(src, BD(0, 3, 3), outs[0], BD(0, 3, 3), *tbl, ws[0], 0, m, **kw)
    Ev.Synchronize()
    ref = z["limit_out6"]
    for k in range(nout):
        # every output within 1e-5 x diag of CpuEvaluator (no scaling); the float table
        # applied in double is reported beside it
        f64 = np.zeros(m * 3)
        oracle.eval_stencils(z["positions"].ravel(), (0, 3, 3), [f64], [(0, 3, 3)],
                             z["limit_sizes"], z["limit_offsets"], z["limit_indices"],
                             [z["limit_" + names[k]]], fp64=True)
        gate(f"{os.path.basename(path)[:-4]} limit {nout} outputs", k, host(outs[k]),
             ref[k].ravel(), f64, diag, all_vs_cpu=True)
    for k in range(nout, 6):
        assert float(host(outs[k]).max()) == 0.0  # not requested: untouched


@pytest.mark.gpu
def test_start_end_subrange_writes_absolute_positions():
    """[start, end) writes destination elements start..end-1 (osd/cudaKernel.cu:85-98)."""
    torch = torch_cuda()
    Ev, BD = _ev()
    z = np.load(FIXTURES[0])
    n = len(z["sizes"])
    start, end = n // 3, n // 3 + 1000
    tbl = [dev(z[k]) for k in ("sizes", "offsets", "indices", "weights")]
    out = torch.full((n * 3,), -7.0, device="cuda")
    assert Ev.EvalStencils(dev(z["positions"].ravel()), BD(0, 3, 3), out, BD(0, 3, 3), *tbl,
                           start, end)
    Ev.Synchronize()
    o = host(out).reshape(n, 3)
    ref = np.full((n, 3), -7.0, np.float32)
    oracle.eval_stencils(z["positions"].ravel(), (0, 3, 3), [ref.reshape(-1)], [(0, 3, 3)],
                         z["sizes"], z["offsets"], z["indices"], [z["weights"]], start, end)
    assert np.all(o[:start] == -7.0) and np.all(o[end:] == -7.0)
    assert max_err(o[start:end], ref[start:end]) <= REL_TOL * bbox_diag(z["positions"])


def _random_table(rng, n, ncv, max_size, big_every=0):
    sizes = rng.integers(1, max_size + 1, n).astype(np.int32)
    if big_every:
        sizes[::big_every] = rng.integers(100, 366, len(sizes[::big_every]))
    offsets = np.zeros(n, np.int32)
    np.cumsum(sizes[:-1], out=offsets[1:])
    nnz = int(sizes.sum())
    idx = rng.integers(0, ncv, nnz).astype(np.int32)
    w = rng.uniform(-0.2, 1.0, nnz).astype(np.float32)
    return sizes, offsets, idx, w


@pytest.mark.gpu
@pytest.mark.parametrize("length", [1, 2, 3, 4, 5, 8, 12, 33])
def test_random_tables_all_lengths_and_pole_sized_stencils(length):
    """Any primvar width (including > 32) and stencils as large as a valence-360 pole."""
    torch = torch_cuda()
    Ev, BD = _ev()
    rng = np.random.default_rng(length)
    ncv, n = 5000, 20000
    sizes, offsets, idx, w = _random_table(rng, n, ncv, 20, big_every=97)
    stride = length + 2
    src = rng.uniform(-1, 1, ncv * stride).astype(np.float32)
    ref = np.zeros(n * length, np.float32)
    oracle.eval_stencils(src, (1, length, stride), [ref], [(0, length, length)], sizes,
                         offsets, idx, [w], threads=8)
    out = torch.zeros(n * length, device="cuda")
    assert Ev.EvalStencils(dev(src), BD(1, length, stride), out, BD(0, length, length),
                           dev(sizes), dev(offsets), dev(idx), dev(w), 0, n)
    Ev.Synchronize()
    # float rounding bound per stencil: a few ulps of sum_j |w_j| max|x| (|x| <= 1)
    absw = np.zeros(n)
    np.add.at(absw, np.repeat(np.arange(n), sizes), np.abs(w))
    bound = np.repeat(4 * 6e-8 * sizes * absw + 1e-7, length)
    assert np.all(np.abs(host(out).astype(np.float64) - ref) <= bound)


@pytest.mark.gpu
@pytest.mark.parametrize("layout", ["reversed_blocks", "gapped", "misaligned_views"])
def test_non_factory_table_layouts(layout):
    """Tables the factories never produce still evaluate correctly: stencil entry blocks
    stored in reverse order (offsets not monotone), gaps between blocks, and table pointers
    that are not 16-byte aligned (sub-array views)."""
    torch = torch_cuda()
    Ev, BD = _ev()
    z = np.load(FIXTURES[0])
    sizes, offsets, idx, w = z["sizes"], z["offsets"], z["indices"], z["weights"]
    n = len(sizes)
    if layout == "reversed_blocks":
        order = np.arange(n)[::-1]
        new_off = np.zeros(n, np.int32)
        new_off[order] = np.concatenate([[0], np.cumsum(sizes[order])[:-1]]).astype(np.int32)
        gather = np.concatenate([np.arange(offsets[i], offsets[i] + sizes[i]) for i in order])
        offsets, idx, w = new_off, idx[gather], w[gather]
    elif layout == "gapped":
        gap = 3
        new_off = (offsets + gap * np.arange(n)).astype(np.int32)
        idx2 = np.zeros(len(idx) + gap * n, np.int32)
        w2 = np.full(len(idx) + gap * n, np.nan, np.float32)  # gap entries must never be read
        for i in range(n):
            idx2[new_off[i]:new_off[i] + sizes[i]] = idx[offsets[i]:offsets[i] + sizes[i]]
            w2[new_off[i]:new_off[i] + sizes[i]] = w[offsets[i]:offsets[i] + sizes[i]]
        offsets, idx, w = new_off, idx2, w2
    tbl = [dev(a) for a in (sizes, offsets, idx, w)]
    if layout == "misaligned_views":
        # one extra leading element, then a view starting at element 1 (4-byte aligned only)
        tbl = [dev(np.concatenate([a[:1], a]))[1:] for a in (sizes, offsets, idx, w)]
    out = torch.zeros(n * 3, device="cuda")
    assert Ev.EvalStencils(dev(z["positions"].ravel()), BD(0, 3, 3), out, BD(0, 3, 3), *tbl,
                           0, n)
    Ev.Synchronize()
    assert max_err(host(out), z["out3"]) <= REL_TOL * bbox_diag(z["positions"])


@pytest.mark.gpu
@pytest.mark.parametrize("outputs", [("P", "du", "dv"), ("P",), ("du", "dv")])
def test_device_table_random_location_limit_stencils(outputs):
    """A limit table at random locations gets a locality-sorted evaluation order inside the
    device table; results must land in the caller's order for every output subset."""
    torch = torch_cuda()
    from opensubdiv_gb300 import shapes, topology
    from opensubdiv_gb300.evaluator import GB300StencilTable
    Ev, BD = _ev()
    cage = shapes.torus(48, 24, tri_fraction=0.05, crease_fraction=0.02, seed=9)
    face, u, v = shapes.uniform_locations(cage, 20000, seed=10)
    lt = topology.UniformRefiner(cage, 2).limit_stencil_table(face, u, v)
    m = len(lt["sizes"])
    table = GB300StencilTable.Create(lt["sizes"], lt["offsets"], lt["indices"], lt["weights"],
                                     lt["du_weights"], lt["dv_weights"])
    src = np.random.default_rng(1).uniform(-1, 1, cage.num_vertices * 8).astype(np.float32)
    d = BD(0, 8, 8)
    outs = {k: torch.zeros(m * 8, device="cuda") for k in ("P", "du", "dv")}
    kw = {}
    for k in ("du", "dv"):
        if k in outputs:
            kw[k], kw[k + "Desc"] = outs[k], d
    dst = outs["P"] if "P" in outputs else None
    assert Ev.EvalStencilsTable(dev(src), d, dst, d if dst is not None else None, table, **kw)
    Ev.Synchronize()
    refs = [np.zeros(m * 8, np.float32) for _ in range(3)]
    oracle.eval_stencils(src, (0, 8, 8), refs, [(0, 8, 8)] * 3, lt["sizes"], lt["offsets"],
                         lt["indices"], [lt["weights"], lt["du_weights"], lt["dv_weights"]],
                         threads=4)
    for k, name in enumerate(("P", "du", "dv")):
        got = host(outs[name])
        if name in outputs:
            A = oracle.stencil_abs_scale(src, (0, 8, 8), lt["sizes"], lt["offsets"],
                                         lt["indices"], [lt["weights"], lt["du_weights"],
                                                         lt["dv_weights"]][k])
            assert np.all(np.abs(got - refs[k]) <= 1e-6 * np.maximum(A, 1.0)), name
        else:
            assert float(np.abs(got).max()) == 0.0


@pytest.mark.gpu
def test_device_status_word_is_clear_after_runs():
    from opensubdiv_gb300 import _lib
    assert _lib.load().GB300GetDeviceStatus() == 0


@pytest.mark.gpu
def test_invalid_requests_return_false_and_empty_ranges_are_noops():
    torch = torch_cuda()
    Ev, BD = _ev()
    z = np.load(FIXTURES[0])
    tbl = [dev(z[k]) for k in ("sizes", "offsets", "indices", "weights")]
    src = dev(z["positions"].ravel())
    out = torch.zeros(30, device="cuda")
    # mismatched lengths: CpuEvaluator returns false (osd/cpuEvaluator.cpp:46-47)
    assert not Ev.EvalStencils(src, BD(0, 3, 3), out, BD(0, 4, 4), *tbl, 0, 10)
    # stride smaller than length
    assert not Ev.EvalStencils(src, BD(0, 3, 2), out, BD(0, 3, 3), *tbl, 0, 10)
    # end <= start is a successful no-op
    assert Ev.EvalStencils(src, BD(0, 3, 3), out, BD(0, 3, 3), *tbl, 5, 5)
    Ev.Synchronize()
    assert float(host(out).max()) == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("length,stride,offset", [(3, 3, 0), (5, 7, 2), (8, 9, 1), (1, 1, 0),
                                                   (12, 12, 0), (11, 13, 3), (16, 16, 0)])
def test_device_table_unaligned_rows_on_a_large_table(length, stride, offset):
    """Device tables of >= 1M entries gather unaligned source rows from a padded copy (rows of
    4, 8, 12 or 16 floats, gathered with vector loads): results must be bit-identical to the
    raw entry point (which gathers in place) and match the oracle."""
    torch = torch_cuda()
    from opensubdiv_gb300 import shapes
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300Evaluator as Ev
    from opensubdiv_gb300.evaluator import GB300StencilTable
    from opensubdiv_gb300.topology import UniformRefiner
    cage = shapes.torus(96, 48, tri_fraction=0.05, crease_fraction=0.02, seed=8)
    r = UniformRefiner(cage, 3).stencil_table()
    n, ncv = len(r["sizes"]), cage.num_vertices
    assert len(r["indices"]) >= 1 << 20
    rng = np.random.default_rng(length)
    src = rng.uniform(-1, 1, ncv * stride + offset).astype(np.float32)
    t = GB300StencilTable.Create(r["sizes"], r["offsets"], r["indices"], r["weights"])
    sd, dd = BD(offset, length, stride), BD(0, length, length)
    a = torch.zeros(n * length, device="cuda")
    b = torch.zeros(n * length, device="cuda")
    s = dev(src)
    assert Ev.EvalStencilsTable(s, sd, a, dd, t)
    # the raw entry point over the table's own device arrays (entries sorted per stencil)
    assert Ev.EvalStencils(s, sd, b, dd, t.GetSizesBuffer(), t.GetOffsetsBuffer(),
                           t.GetIndicesBuffer(), t.GetWeightsBuffer(), 0, n)
    Ev.Synchronize()
    assert torch.equal(a, b)
    out = np.zeros(n * length, np.float32)
    oracle.eval_stencils(src, (offset, length, stride), [out], [(0, length, length)],
                         r["sizes"], r["offsets"], r["indices"], [r["weights"]], threads=8)
    bound = 1e-6 * oracle.stencil_abs_scale(src, (offset, length, stride), r["sizes"],
                                            r["offsets"], r["indices"], r["weights"]) + 1e-6
    assert np.all(np.abs(host(a) - out) <= bound)
