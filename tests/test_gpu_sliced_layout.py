"""Device stencil tables evaluate through their sliced layout (32-stencil slices stored
entry-major, built on the device at creation): edge cases of that layout against the oracle.

Covered: stencil counts that leave a partial last slice (1, 31, 33, ...), empty stencils
between and after others, tables without any entry, slices far wider than a staging stage
(valence-360 poles: the kernel's unstaged path), the locality order of scattered tables
(n >= 4096), every output count 1-6 with output descriptors of every store width, and
primvar widths 1-33 including the 9-12 wide single pass.  Tolerance: the rounding bound of
two summation orders of the same entries (see _bound).
"""
import numpy as np
import pytest

import oracle
from gpu_util import dev, host, torch_cuda


def _api():
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300StencilTable)
    return Ev, BD, GB300StencilTable


def _table(rng, n, ncv, max_size, empty_every=0, pole_every=0, scatter=False):
    sizes = rng.integers(1, max_size + 1, n).astype(np.int32)
    if pole_every:
        sizes[::pole_every] = rng.integers(100, 366, len(sizes[::pole_every]))
    if empty_every:
        sizes[::empty_every] = 0
        sizes[-1] = 0
    offsets = np.zeros(n, np.int32)
    np.cumsum(sizes[:-1], out=offsets[1:])
    nnz = int(sizes.sum())
    if scatter:
        # each stencil reads a cluster around a random centre: consecutive stencils jump
        centre = np.repeat(rng.integers(0, ncv, n), sizes)
        idx = ((centre + rng.integers(-8, 9, nnz)) % ncv).astype(np.int32)
    else:
        idx = rng.integers(0, ncv, nnz).astype(np.int32)
    ws = [rng.uniform(-0.2, 1.0, nnz).astype(np.float32) for _ in range(6)]
    return sizes, offsets, idx, ws


def _bound(src, desc, sizes, offsets, idx, w):
    """Per element: device tables hold each stencil's entries sorted by control index, so
    the sum runs in another order than the oracle's; each order's rounding error is at most
    (size - 1) u sum_j |w_j x_j| (u = 2^-24, recursive summation), so they differ by at most
    twice that (plus 2 ulps for the fused multiply-adds)."""
    a = oracle.stencil_abs_scale(src, desc, sizes, offsets, idx, w).reshape(len(sizes), -1)
    u = 2.0 ** -24
    return (2.0 * np.maximum(sizes, 1)[:, None] + 2.0) * u * a + 1e-7


def _check(torch, n, ncv, length, sizes, offsets, idx, ws, nout=1, seed=0, src_desc=None,
           dst_descs=None):
    Ev, BD, Table = _api()
    rng = np.random.default_rng(seed)
    sd = src_desc or (0, length, length)
    src = rng.uniform(-1, 1, ncv * sd[2] + sd[0]).astype(np.float32)
    dds = dst_descs or [(0, length, length)] * nout
    table = Table.Create(sizes, offsets, idx, *ws[:nout])
    outs = [torch.zeros(n * d[2] + d[0], device="cuda") for d in dds]
    keys = ("du", "dv", "duu", "duv", "dvv")
    kw = {}
    for k in range(1, nout):
        kw[keys[k - 1]], kw[keys[k - 1] + "Desc"] = outs[k], BD(*dds[k])
    assert Ev.EvalStencilsTable(dev(src), BD(*sd), outs[0], BD(*dds[0]), table, **kw)
    Ev.Synchronize()
    for k in range(nout):
        ref = np.zeros(n * dds[k][2] + dds[k][0], np.float32)
        oracle.eval_stencils(src, sd, [ref], [dds[k]], sizes, offsets, idx, [ws[k]], threads=8)
        got = host(outs[k]).reshape(-1)
        off, ln, st = dds[k]
        g = got[off: off + n * st].reshape(n, st)[:, :ln].astype(np.float64)
        r = ref[off: off + n * st].reshape(n, st)[:, :ln]
        b = _bound(src, sd, sizes, offsets, idx, ws[k])
        ratio = float((np.abs(g - r) / b).max(initial=0.0))
        assert ratio <= 1.0, (k, ratio)
        # elements outside each output row's [offset, offset + length) stay untouched
        rest = got.copy()
        rest[off: off + n * st].reshape(n, st)[:, :ln] = 0.0
        assert float(np.abs(rest).max(initial=0.0)) == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 31, 32, 33, 257, 4095, 4097])
def test_partial_last_slice_and_small_tables(n):
    torch = torch_cuda()
    rng = np.random.default_rng(n)
    sizes, offsets, idx, ws = _table(rng, n, 700, 20)
    _check(torch, n, 700, 8, sizes, offsets, idx, ws, seed=n)


@pytest.mark.gpu
@pytest.mark.parametrize("length", [1, 2, 3, 4, 8, 11, 12, 33])
def test_empty_and_pole_stencils(length):
    """Empty stencils (every 7th and the last) write zeros; valence-360 poles make slices
    wider than a stage, which the kernel reads straight from global memory."""
    torch = torch_cuda()
    rng = np.random.default_rng(100 + length)
    n, ncv = 20011, 5000
    sizes, offsets, idx, ws = _table(rng, n, ncv, 20, empty_every=7, pole_every=97)
    _check(torch, n, ncv, length, sizes, offsets, idx, ws, seed=length)


@pytest.mark.gpu
def test_table_without_entries():
    torch = torch_cuda()
    Ev, BD, Table = _api()
    n = 100
    sizes = np.zeros(n, np.int32)
    offsets = np.zeros(n, np.int32)
    table = Table.Create(sizes, offsets, np.zeros(0, np.int32), np.zeros(0, np.float32))
    from opensubdiv_gb300.evaluator import last_error
    out = torch.full((n * 4,), 5.0, device="cuda")
    ok = Ev.EvalStencilsTable(dev(np.ones(40, np.float32)), BD(0, 4, 4), out, BD(0, 4, 4),
                              table)
    assert ok, last_error()
    Ev.Synchronize()
    assert float(host(out).max()) == 0.0 and float(host(out).min()) == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("nout", [1, 2, 3, 4, 5, 6])
def test_scattered_table_every_output_count_and_store_width(nout):
    """A scattered table (locality order on the device) with 1-6 outputs whose descriptors
    take 256-bit (stride 8), 128-bit (stride 12, offset 4) and scalar (stride 9, offset 1)
    stores."""
    torch = torch_cuda()
    rng = np.random.default_rng(200 + nout)
    n, ncv = 12000, 3000
    sizes, offsets, idx, ws = _table(rng, n, ncv, 24, empty_every=53, scatter=True)
    descs = [(0, 8, 8), (4, 8, 12), (1, 8, 9), (0, 8, 8), (4, 8, 12), (1, 8, 9)][:nout]
    _check(torch, n, ncv, 8, sizes, offsets, idx, ws, nout=nout, seed=nout, dst_descs=descs)


@pytest.mark.gpu
@pytest.mark.parametrize("src_desc", [(0, 8, 8), (4, 8, 12), (0, 10, 12), (2, 6, 9), (0, 3, 4),
                                      (4, 4, 8)])
def test_source_layouts(src_desc):
    """Source rows gathered with 256-bit, 128-bit, 12-wide, scalar and 4-column (rows of at
    most 4 floats) loads."""
    torch = torch_cuda()
    rng = np.random.default_rng(300 + src_desc[2])
    n, ncv = 9000, 2500
    sizes, offsets, idx, ws = _table(rng, n, ncv, 18, empty_every=41)
    ln = src_desc[1]
    _check(torch, n, ncv, ln, sizes, offsets, idx, ws, nout=3, seed=7, src_desc=src_desc,
           dst_descs=[(0, ln, ln)] * 3)
