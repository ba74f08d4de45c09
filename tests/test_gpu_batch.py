"""Batched EvalStencils (one persistent launch over many meshes) through the C ABI.

Every job of a batch must produce what one plain EvalStencilsTable call per mesh produces:
bit-identical where a job runs one stencil per thread (same entries, same order, same fused
multiply-adds), within float rounding of the oracle where large stencils are evaluated one per
warp.  Covers uneven Catmull-Clark / Loop meshes at levels 1-4 with 3-12 primvars, descriptor
offsets inside interleaved buffers, empty tables, tables with large stencils, the CUDA-graph
replay, the autotuner and the device status word.
"""
import numpy as np
import pytest

import oracle
from gpu_util import dev, host, torch_cuda


def _population(n=24, cv_max=3000, seed=11):
    from opensubdiv_gb300 import workloads
    return workloads.batch_population(n_meshes=n, cv_min=60, cv_max=cv_max, seed=seed)


def _big_stencil_table(n_stencils, n_cv, rng, lo=80, hi=400):
    sizes = rng.integers(lo, hi, n_stencils).astype(np.int32)
    offsets = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int32)
    idx = rng.integers(0, n_cv, int(sizes.sum())).astype(np.int32)
    w = (rng.random(int(sizes.sum())) / lo).astype(np.float32)
    return dict(sizes=sizes, offsets=offsets, indices=idx, weights=w)


def _oracle_out(table, src, length, n_cv):
    n = len(table["sizes"])
    out = np.zeros(n * length, np.float32)
    oracle.eval_stencils(src, (0, length, length), [out], [(0, length, length)],
                         table["sizes"], table["offsets"], table["indices"], [table["weights"]],
                         threads=4)
    return out


def _abs_bound(table, src, length):
    """Per-output bound for a reordered float sum: 1e-6 x sum_j |w_j x_j| + 1e-6."""
    return 1e-6 * oracle.stencil_abs_scale(src, (0, length, length), table["sizes"],
                                           table["offsets"], table["indices"],
                                           table["weights"]) + 1e-6


def _plain(torch, tables, srcs, descs_s, dsts_plain, descs_d):
    from opensubdiv_gb300.evaluator import GB300Evaluator as Ev
    for t, s, sd, d, dd in zip(tables, srcs, descs_s, dsts_plain, descs_d):
        assert Ev.EvalStencilsTable(s, sd, d, dd, t)
    Ev.Synchronize()


@pytest.mark.gpu
def test_batch_matches_plain_calls_and_oracle():
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD
    from opensubdiv_gb300.evaluator import GB300StencilBatch, GB300StencilTable
    pop = _population()
    rng = np.random.default_rng(4)
    tables, srcs, sd, dsts, dsts_plain, dd, meta = [], [], [], [], [], [], []
    for k, m in enumerate(pop):
        L = m["length"]
        tables.append(GB300StencilTable.Create(**m["table"]))
        n = len(m["table"]["sizes"])
        if k % 3 == 1:
            # primvar at an offset inside a wider interleaved buffer, on both sides
            pad = 5
            wide = rng.uniform(-1, 1, (m["n_cv"], L + pad)).astype(np.float32)
            wide[:, 2:2 + L] = m["src"].reshape(-1, L)
            srcs.append(dev(wide.ravel()))
            sd.append(BD(2, L, L + pad))
            dsts.append(torch.full((n * (L + 3),), 7.0, device="cuda"))
            dsts_plain.append(torch.full((n * (L + 3),), 7.0, device="cuda"))
            dd.append(BD(1, L, L + 3))
        else:
            srcs.append(dev(m["src"]))
            sd.append(BD(0, L, L))
            dsts.append(torch.zeros(n * L, device="cuda"))
            dsts_plain.append(torch.zeros(n * L, device="cuda"))
            dd.append(BD(0, L, L))
        meta.append(m)
    batch = GB300StencilBatch(list(zip(tables, srcs, sd, dsts, dd)))
    cfg = batch.GetConfig()
    assert cfg["num_tiles"] > len(pop)
    batch.Eval()
    _plain(torch, tables, srcs, sd, dsts_plain, dd)
    for k, m in enumerate(meta):
        L, n = m["length"], len(m["table"]["sizes"])
        g = host(dsts[k])
        p = host(dsts_plain[k])
        assert np.array_equal(g, p), f"job {k} ({m['name']}) differs from the plain call"
        out = g.reshape(n, dd[k].stride)[:, dd[k].offset:dd[k].offset + L].ravel()
        ref = _oracle_out(m["table"], m["src"], L, m["n_cv"])
        assert np.all(np.abs(out - ref) <= _abs_bound(m["table"], m["src"], L)), m["name"]
        if dd[k].stride > L:  # untouched padding lanes keep their contents
            pad = g.reshape(n, dd[k].stride)
            assert np.all(pad[:, 0] == 7.0) and np.all(pad[:, L + 1:] == 7.0)
    assert batch.GetDeviceStatus() == 0


@pytest.mark.gpu
def test_batch_graph_replay_tune_and_deformation():
    """Frames: deform the sources in place, replay the captured graph, compare with plain
    calls; then autotune and check the tuned batch still matches."""
    torch = torch_cuda()
    from opensubdiv_gb300 import workloads
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD
    from opensubdiv_gb300.evaluator import GB300StencilBatch, GB300StencilTable
    pop = _population(n=16, cv_max=2000, seed=12)
    tables = [GB300StencilTable.Create(**m["table"]) for m in pop]
    base = [dev(m["src"]) for m in pop]
    srcs = [b.clone() for b in base]
    descs = [BD(0, m["length"], m["length"]) for m in pop]
    dsts = [torch.zeros(len(m["table"]["sizes"]) * m["length"], device="cuda") for m in pop]
    plain = [torch.zeros_like(d) for d in dsts]
    batch = GB300StencilBatch(list(zip(tables, srcs, descs, dsts, descs)))
    for frame in range(3):
        for b, s, m in zip(base, srcs, pop):
            s.copy_(workloads.deform(b, m["phase"], frame))
        batch.EvalGraph()
        _plain(torch, tables, srcs, descs, plain, descs)
        for d, p in zip(dsts, plain):
            assert torch.equal(d, p), f"frame {frame}"
    batch.Tune(iterations=2)
    cfg = batch.GetConfig()
    assert cfg["tile_stencils"] in (64, 128, 256) and cfg["ctas_per_sm"] in (1, 2, 3)
    for d in dsts:
        d.zero_()
    batch.EvalGraph()
    torch.cuda.synchronize()
    for d, p in zip(dsts, plain):
        assert torch.equal(d, p)
    # a second batch with the same work histogram picks up the tuned configuration
    again = GB300StencilBatch(list(zip(tables, srcs, descs, dsts, descs)))
    assert again.GetConfig() == cfg
    assert batch.GetDeviceStatus() == 0


@pytest.mark.gpu
def test_batch_large_stencils_warp_mode_and_empty_jobs():
    """Jobs whose mean stencil size exceeds the warp threshold run one stencil per warp
    (shuffle reduction): within float rounding of the oracle.  Empty tables are no-ops."""
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD
    from opensubdiv_gb300.evaluator import GB300StencilBatch, GB300StencilTable
    rng = np.random.default_rng(21)
    jobs, refs = [], []
    keep = []
    for k, (ns, ncv, L, lo, hi) in enumerate([(700, 5000, 3, 80, 400), (3000, 20000, 8, 100, 300),
                                              (50, 300, 12, 4, 20), (500, 3000, 6, 70, 100),
                                              (0, 10, 4, 1, 2),
                                              (1, 40, 5, 300, 301)]):
        table = _big_stencil_table(ns, ncv, rng, lo, hi) if ns else dict(
            sizes=np.zeros(0, np.int32), offsets=np.zeros(0, np.int32),
            indices=np.zeros(0, np.int32), weights=np.zeros(0, np.float32))
        src = rng.uniform(-1, 1, ncv * L).astype(np.float32)
        t = GB300StencilTable.Create(**table)
        s = dev(src)
        d = torch.full((max(ns, 1) * L,), 3.0, device="cuda")
        keep.append((t, s, d))
        jobs.append((t, s, BD(0, L, L), d, BD(0, L, L)))
        refs.append((table, src, L, ns))
    batch = GB300StencilBatch(jobs)
    assert batch.GetConfig()["warp_threshold"] == 64
    batch.Eval()
    torch.cuda.synchronize()
    for (t, s, d), (table, src, L, ns) in zip(keep, refs):
        g = host(d)
        if ns == 0:
            assert np.all(g == 3.0)
            continue
        ref = _oracle_out(table, src, L, len(src) // L)
        assert np.all(np.abs(g - ref) <= _abs_bound(table, src, L))
    assert batch.GetDeviceStatus() == 0


@pytest.mark.gpu
def test_batch_invalid_requests():
    torch = torch_cuda()
    from opensubdiv_gb300 import _lib
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD
    from opensubdiv_gb300.evaluator import GB300Error, GB300StencilBatch, GB300StencilTable
    m = _population(n=1, cv_max=200, seed=3)[0]
    t = GB300StencilTable.Create(**m["table"])
    s = dev(m["src"])
    d = torch.zeros(len(m["table"]["sizes"]) * m["length"], device="cuda")
    L = m["length"]
    with pytest.raises(ValueError):
        GB300StencilBatch([(t, s, BD(0, L, L), d, BD(0, L - 1, L))])
    with pytest.raises(GB300Error):
        GB300StencilBatch([])
    lib = _lib.load()
    assert lib.GB300StencilBatchEval(None, None) == 1
    assert lib.GB300StencilBatchEvalGraph(None, None) == 1


@pytest.mark.gpu
def test_batch_mixed_padded_widths_with_odd_row_counts():
    """Unaligned jobs of every padded width (rows of 8, 12 and 16 floats) with an odd number of
    source rows, side by side in one batch: each job's padded region starts on a 64-byte
    boundary, so the 256-bit and 128-bit gathers stay aligned; results equal plain calls."""
    torch = torch_cuda()
    from opensubdiv_gb300 import shapes, topology
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD
    from opensubdiv_gb300.evaluator import GB300StencilBatch, GB300StencilTable
    cage = shapes.torus(7, 5, tri_fraction=0.1, seed=3)
    ncv = cage.num_vertices
    assert ncv % 2 == 1
    t = topology.UniformRefiner(cage, 2).stencil_table()
    table = GB300StencilTable.Create(**t)
    n = len(t["sizes"])
    rng = np.random.default_rng(12)
    widths = [9, 3, 11, 5, 10, 13, 7, 6, 15, 12, 14]
    srcs, dsts, plain, descs = [], [], [], []
    for L in widths:
        srcs.append(dev(rng.uniform(-1, 1, ncv * L).astype(np.float32)))
        dsts.append(torch.zeros(n * L, device="cuda"))
        plain.append(torch.zeros(n * L, device="cuda"))
        descs.append(BD(0, L, L))
    batch = GB300StencilBatch([(table, s, d, o, d) for s, o, d in zip(srcs, dsts, descs)])
    batch.Eval()
    _plain(torch, [table] * len(widths), srcs, descs, plain, descs)
    for L, a, b in zip(widths, dsts, plain):
        assert torch.equal(a, b), L
    assert batch.GetDeviceStatus() == 0


@pytest.mark.gpu
def test_batch_of_only_wide_jobs():
    """Every job 9-12 floats wide (aligned and padded rows): the general launch has no jobs and
    the 12-wide launch does all the work; graph replay included; results equal plain calls."""
    torch = torch_cuda()
    from opensubdiv_gb300 import shapes, topology
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD
    from opensubdiv_gb300.evaluator import GB300StencilBatch, GB300StencilTable
    cage = shapes.torus(9, 7, tri_fraction=0.1, seed=5)
    t = topology.UniformRefiner(cage, 2).stencil_table()
    table = GB300StencilTable.Create(**t)
    n, ncv = len(t["sizes"]), cage.num_vertices
    rng = np.random.default_rng(13)
    widths = [(12, 12), (9, 9), (10, 12), (11, 11), (12, 16)]
    srcs, dsts, plain, sds, dds = [], [], [], [], []
    for L, stride in widths:
        srcs.append(dev(rng.uniform(-1, 1, ncv * stride).astype(np.float32)))
        dsts.append(torch.zeros(n * L, device="cuda"))
        plain.append(torch.zeros(n * L, device="cuda"))
        sds.append(BD(0, L, stride))
        dds.append(BD(0, L, L))
    batch = GB300StencilBatch([(table, s, sd, o, dd)
                               for s, sd, o, dd in zip(srcs, sds, dsts, dds)])
    assert batch.GetConfig()["num_tiles"] > 0
    batch.EvalGraph()
    _plain(torch, [table] * len(widths), srcs, sds, plain, dds)
    for (L, stride), a, b in zip(widths, dsts, plain):
        assert torch.equal(a, b), (L, stride)
    assert batch.GetDeviceStatus() == 0


@pytest.mark.gpu
def test_sliced_and_far_layout_batches_agree_bit_for_bit():
    """A batch whose tables all carry their sliced layout runs the sliced tiles (three
    launches: any width, at most 4 floats, 9-12 floats); one table without stencils (no
    sliced layout) switches the same jobs to the Far-layout tiles.  Both must write identical
    bits."""
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD
    from opensubdiv_gb300.evaluator import GB300StencilBatch, GB300StencilTable
    pop = _population(n=20, cv_max=2500, seed=21)
    tables = [GB300StencilTable.Create(**m["table"]) for m in pop]
    srcs = [dev(m["src"]) for m in pop]
    descs = [BD(0, m["length"], m["length"]) for m in pop]
    a = [torch.zeros(len(m["table"]["sizes"]) * m["length"], device="cuda") for m in pop]
    b = [torch.zeros_like(x) for x in a]
    sliced = GB300StencilBatch(list(zip(tables, srcs, descs, a, descs)))
    # a table without stencils has no sliced layout
    empty = GB300StencilTable.Create(np.zeros(0, np.int32), np.zeros(0, np.int32),
                                     np.zeros(0, np.int32), np.zeros(0, np.float32))
    e_out = torch.full((3,), 9.0, device="cuda")
    far = GB300StencilBatch(list(zip(tables, srcs, descs, b, descs)) +
                            [(empty, srcs[0], BD(0, 3, 3), e_out, BD(0, 3, 3))])
    sliced.Eval()
    far.Eval()
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    assert float(e_out.min()) == 9.0 and float(e_out.max()) == 9.0
    lengths = {m["length"] for m in pop}
    assert lengths & {3, 4} and lengths & {9, 10, 11, 12}
