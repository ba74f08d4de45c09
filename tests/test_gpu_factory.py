"""The GPU stencil-table factory (GB300StencilTableFactoryCreate, GB300StencilTableComposeRows)
against the reference's own tables and the oracle.

The masks in tests/golden/factory_masks.npz were recorded from Far::PrimvarRefiner; the device
factory must rebuild Far::StencilTableFactory's tables from them bit for bit (entries in Far's
order), and with sorted entries must hold the same stencils.  Compositions over a base table
(limit-stencil and local-point forms) must equal the oracle's restatement bit for bit."""
import numpy as np
import pytest

import oracle
from gpu_util import dev, torch_cuda
from test_factory_oracle import (CHANNELS, GOLDEN, LIMIT, cases, far_table, limit_case,
                                 limit_cases, load_case, same_limit_table, same_table)


def sorted_rows(t):
    """The table with each stencil's entries sorted by control index (stable)."""
    idx = t["indices"].copy()
    w = t["weights"].copy()
    for i, (o, n) in enumerate(zip(t["offsets"], t["sizes"])):
        p = np.argsort(idx[o:o + n], kind="stable")
        idx[o:o + n] = idx[o:o + n][p]
        w[o:o + n] = w[o:o + n][p]
    return dict(sizes=t["sizes"], offsets=t["offsets"], indices=idx, weights=w)


@pytest.mark.gpu
@pytest.mark.parametrize("name", cases())
@pytest.mark.parametrize("tag,inter,ctrl", [("all", True, False), ("last_ctrl", False, True)])
def test_factory_rebuilds_far_tables(name, tag, inter, ctrl):
    torch_cuda()
    from opensubdiv_gb300.evaluator import GB300StencilTableFactory as F
    z = np.load(GOLDEN)
    nc, levels = load_case(z, name)
    far = far_table(z, name, tag)
    t = F.Create(nc, levels, generateIntermediateLevels=inter, generateControlVerts=ctrl,
                 sortEntries=False)
    assert same_table(t.CopyToHost(), far)
    s = F.Create(nc, levels, generateIntermediateLevels=inter, generateControlVerts=ctrl,
                 sortEntries=True)
    assert same_table(s.CopyToHost(), sorted_rows(far))


@pytest.mark.gpu
def test_factory_table_evaluates_like_the_uploaded_far_table():
    """EvalStencils over the factory's table (sorted layout) and over GB300StencilTable.Create
    of Far's arrays: the same device layout, so bit-identical results."""
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300StencilTable, GB300StencilTableFactory as F)
    z = np.load(GOLDEN)
    nc, levels = load_case(z, "torus")
    far = far_table(z, "torus", "all")
    a = F.Create(nc, levels)
    b = GB300StencilTable.Create(far["sizes"], far["offsets"], far["indices"], far["weights"])
    n = a.GetNumStencils()
    src = dev(np.random.default_rng(5).normal(size=nc * 4).astype(np.float32))
    d = BD(0, 4, 4)
    ya = torch.zeros(n * 4, device="cuda")
    yb = torch.zeros(n * 4, device="cuda")
    assert Ev.EvalStencilsTable(src, d, ya, d, a)
    assert Ev.EvalStencilsTable(src, d, yb, d, b)
    torch.cuda.synchronize()
    assert torch.equal(ya, yb)


def _device_base(rng, n_ctrl, n_rows, max_size):
    """A device table in Far's entry order, built by ComposeRows over identity rows: each row
    gets distinct control indices, and some rows an extra entry that cancels one weight to an
    exact 0.0 (zero entries stay in the row, as Far's merges keep them)."""
    from opensubdiv_gb300.evaluator import GB300StencilTable
    ident = np.arange(n_ctrl, dtype=np.int32)
    idt = GB300StencilTable.Create(np.ones(n_ctrl, np.int32), ident, ident,
                                   np.ones(n_ctrl, np.float32))
    off, src, w = [0], [], []
    for _ in range(n_rows):
        q = rng.choice(n_ctrl, int(rng.integers(1, max_size + 1)), replace=False)
        x = rng.normal(size=len(q)).astype(np.float32)
        src += q.tolist()
        w += x.tolist()
        if rng.random() < 0.1:
            j = int(rng.integers(len(q)))
            src.append(int(q[j]))
            w.append(-float(x[j]))
        off.append(len(src))
    b = GB300StencilTable.ComposeRows(idt, np.array(off, np.int64), np.array(src, np.int32),
                                      [np.array(w, np.float32)], sortEntries=False)
    return b, b.CopyToHost()


@pytest.mark.gpu
@pytest.mark.parametrize("nch,append", [(1, False), (3, False), (6, False), (1, True)])
def test_compose_rows_matches_oracle(nch, append):
    """Limit-stencil form (patch CVs x basis weights, 1 / 3 / 6 channels) and the local-point
    append form over a base table whose rows overlap heavily (merges hit existing entries),
    with zero base entries (skipped), zero mask weights, masks longer than a warp and rows
    longer than the 256-entry shared-memory list."""
    torch_cuda()
    from opensubdiv_gb300.evaluator import GB300StencilTable
    rng = np.random.default_rng(100 + nch)
    b, base = _device_base(rng, 400, 3000, 24)
    assert (base["weights"] == 0).any()
    n = 2000
    cnt = rng.integers(1, 21, n)
    cnt[:3] = [60, 200, 40]  # long masks: rows of hundreds of entries
    off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
    src = rng.integers(0, 3000, int(off[-1])).astype(np.int32)
    ws = [rng.normal(size=len(src)).astype(np.float32) for _ in range(nch)]
    zero = rng.random(len(src)) < 0.05
    for w in ws:
        w[zero] = 0.0
    want = oracle.compose_rows(base, off, src, ws, append_base=append)
    assert want["sizes"].max() > 256
    got = GB300StencilTable.ComposeRows(b, off, src, ws, appendBase=append, sortEntries=False)
    h = got.CopyToHost()
    names = ("weights", "du_weights", "dv_weights", "duu_weights", "duv_weights",
             "dvv_weights")
    for k in ("sizes", "offsets", "indices"):
        assert np.array_equal(h[k], want[k]), k
    for c in range(nch):
        assert np.array_equal(h[names[c]].view(np.uint32), want[names[c]].view(np.uint32))


@pytest.mark.gpu
def test_factory_rejects_malformed_masks():
    torch_cuda()
    from opensubdiv_gb300.evaluator import GB300Error, GB300StencilTableFactory as F
    z = np.load(GOLDEN)
    nc, levels = load_case(z, "cube")
    bad = [dict(d) for d in levels]
    bad[2] = dict(bad[2], sources=bad[2]["sources"].copy())
    bad[2]["sources"][5] = nc + 3  # an older level: not allowed with factorized levels
    with pytest.raises(GB300Error):
        F.Create(nc, bad)
    bad[2]["sources"][5] = 1 << 30  # beyond every vertex
    with pytest.raises(GB300Error):
        F.Create(nc, bad)
    # the device is still usable afterwards
    t = F.Create(nc, levels)
    assert t.GetNumStencils() == sum(len(d["offsets"]) - 1 for d in levels)


@pytest.mark.gpu
@pytest.mark.parametrize("name", limit_cases())
def test_limit_pipeline_rebuilds_far_limit_tables(name):
    """The device LimitStencilTableFactory pipeline (GB300LimitStencilTableFactory::Create's
    steps through the C ABI): refined-vertex table, local-point splice, per-location merges with
    Far's basis weights -- bit for bit Far::LimitStencilTableFactory's table."""
    torch_cuda()
    from opensubdiv_gb300.evaluator import GB300StencilTable, GB300StencilTableFactory as F
    rec, far = limit_case(np.load(LIMIT), name)
    cv = F.Create(rec["num_control"], rec["levels"],
                  generateIntermediateLevels=rec["intermediate"], generateControlVerts=True,
                  sortEntries=False)
    if rec["spliced"]:
        o, s, w = rec["local"]
        cv = GB300StencilTable.ComposeRows(cv, o, s, [w], appendBase=True, sortEntries=False)
    o, s, ws = rec["loc"]
    lim = GB300StencilTable.ComposeRows(cv, o, s, ws, sortEntries=False)
    assert same_limit_table(lim.CopyToHost(), far, rec["num_channels"])


@pytest.mark.gpu
def test_composed_scattered_table_evaluates_like_an_uploaded_one():
    """Limit-like stencils at scattered locations (consecutive stencils far apart): the device
    assembly builds the same locality-sorted evaluation layout GB300StencilTable.Create keeps,
    so EvalStencils results are bit-identical to the uploaded copy of the same arrays, and
    within float rounding of the oracle."""
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300StencilTable)
    rng = np.random.default_rng(77)
    b, base = _device_base(rng, 5000, 20000, 12)
    n = 6000
    cnt = np.full(n, 16)
    off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
    # each location reads 16 rows around a random centre: scattered from one stencil to the next
    centre = rng.integers(0, 20000 - 64, n)
    src = (centre[:, None] + rng.integers(0, 64, (n, 16))).astype(np.int32).ravel()
    ws = [rng.normal(size=len(src)).astype(np.float32) for _ in range(3)]
    t = GB300StencilTable.ComposeRows(b, off, src, ws)  # sorted entries + evaluation order
    h = t.CopyToHost()
    u = GB300StencilTable.Create(h["sizes"], h["offsets"], h["indices"], h["weights"],
                                 h["du_weights"], h["dv_weights"])
    L = 4
    x = rng.uniform(-1, 1, 5000 * L).astype(np.float32)
    d = BD(0, L, L)
    outs = [[torch.zeros(n * L, device="cuda") for _ in range(3)] for _ in range(2)]
    for tab, o in zip((t, u), outs):
        assert Ev.EvalStencilsTable(dev(x), d, o[0], d, tab, du=o[1], duDesc=d, dv=o[2],
                                    dvDesc=d)
    torch.cuda.synchronize()
    for a, c in zip(*outs):
        assert torch.equal(a, c)
    ref = [np.zeros(n * L, np.float32) for _ in range(3)]
    oracle.eval_stencils(x, (0, L, L), ref, [(0, L, L)] * 3, h["sizes"], h["offsets"],
                         h["indices"], [h["weights"], h["du_weights"], h["dv_weights"]])
    for a, r in zip(outs[0], ref):
        assert np.abs(a.cpu().numpy() - r).max() <= 1e-4 * max(1.0, np.abs(r).max())


@pytest.mark.gpu
@pytest.mark.parametrize("cage_id", ["torus_creases_L3", "cube_L4", "loop_L3", "pole30_L3"])
def test_factory_on_generator_masks_matches_oracle(cage_id):
    """Larger tables from the host generator's masks (Far::PrimvarRefiner form): the device
    factory equals the oracle's restatement of StencilBuilder's merge bit for bit, for every
    level (intermediate levels kept) and for the last level with control vertices."""
    torch_cuda()
    from opensubdiv_gb300 import shapes, topology
    from opensubdiv_gb300.evaluator import GB300StencilTableFactory as F
    cage, level = {
        "torus_creases_L3": (shapes.torus(64, 32, tri_fraction=0.1, crease_fraction=0.05,
                                          seed=21), 3),
        "cube_L4": (shapes.cube(6, seed=22), 4),
        "loop_L3": (shapes.torus(32, 16, crease_fraction=0.05, seed=23,
                                 scheme=shapes.LOOP), 3),
        "pole30_L3": (shapes.bipyramid(30), 3),
    }[cage_id]
    nc, levels = topology.UniformRefiner(cage, level, stencils=False).factory_masks()
    for inter, ctrl in ((True, False), (False, True)):
        want = oracle.factory_create(nc, levels, intermediate=inter, control=ctrl)
        got = F.Create(nc, levels, generateIntermediateLevels=inter, generateControlVerts=ctrl,
                       sortEntries=False).CopyToHost()
        assert same_table(got, want), (inter, ctrl)


def _random_levels(rng, nc, rows, fan=6, same_level=0.3, zero=0.05):
    """Random masks: each row names sources of the previous level (or control vertices) and,
    with probability `same_level`, earlier rows of its own level, so dependency chains run
    several waves deep; some weights are 0 (dropped) and some rows end up empty."""
    levels, first, prev_first, prev_n = [], nc, 0, nc
    for n in rows:
        off, src, w = [0], [], []
        for r in range(n):
            k = int(rng.integers(0, fan + 1))
            for _ in range(k):
                if r > 0 and rng.random() < same_level:
                    src.append(first + int(rng.integers(0, r)))
                else:
                    src.append(prev_first + int(rng.integers(0, prev_n)))
                w.append(0.0 if rng.random() < zero else float(rng.normal()))
            off.append(len(src))
        levels.append(dict(offsets=np.array(off, np.int64), sources=np.array(src, np.int32),
                           weights=np.array(w, np.float32)))
        prev_first, prev_n, first = first, n, first + n
    return levels


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_factory_random_masks_match_oracle(seed):
    """Synthetic masks with deep same-level chains (many dependency waves), zero weights,
    empty rows, an empty level and mixed row lengths: device factory == oracle, bit for bit;
    a factory with no levels gives one identity stencil per control vertex."""
    torch_cuda()
    from opensubdiv_gb300.evaluator import GB300StencilTableFactory as F
    rng = np.random.default_rng(seed)
    nc = 50
    levels = _random_levels(rng, nc, [200, 400, 900, 0] if seed == 2 else [200, 400, 900])
    for inter, ctrl in ((True, False), (False, True)):
        want = oracle.factory_create(nc, levels, intermediate=inter, control=ctrl)
        got = F.Create(nc, levels, generateIntermediateLevels=inter, generateControlVerts=ctrl,
                       sortEntries=False).CopyToHost()
        assert same_table(got, want), (inter, ctrl)
    ident = F.Create(nc, [], generateControlVerts=True, sortEntries=False).CopyToHost()
    assert np.array_equal(ident["sizes"], np.ones(nc, np.int32))
    assert np.array_equal(ident["indices"], np.arange(nc, dtype=np.int32))
    assert np.array_equal(ident["weights"], np.ones(nc, np.float32))
