"""Bfr tessellation and evaluation of whole meshes on the device (GB300TessellationCount /
GB300TessellationGenerate + GB300PatchTableEval) against the reference's Bfr.

* Patterns: the device tessellation of every case of the reference's Bfr::Tessellation sweep
  (tests/golden/bfr_tess_patterns.npz) -- counts, coords bit for bit, facets exactly -- through
  per-face rate runs, and the shared uniform-rate patterns for faces of 3..13 sides against the
  oracle (pinned to the same sweep by tests/test_bfr_oracle.py).
* Meshes: the reference's tessellate-and-evaluate loop (tests/golden/bfr_<mesh>_*.npz): coords,
  facets with mesh-wide indices, located PatchCoords (handles exact, (s,t) bit for bit) and the
  six evaluated outputs.  P, Du, Dv and the second derivatives are held to the reference's own
  Bfr-versus-Far tolerances against Bfr::Surface::Evaluate, and to the accuracy gate
  (tests/gpu_util.py) against the oracle's evaluation of the same Far table.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from gpu_util import bbox_diag, dev, gate, host, torch_cuda
from test_bfr_oracle import STENCIL_MESHES, STENCILS, oracle_point_stencils, point_base

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MESHES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "bfr_*.npz"))
                if not p.endswith(("bfr_tess_patterns.npz", "bfr_share.npz", "bfr_stencils.npz")))


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.int32)


def bfr_tolerances(positions):
    """regression/bfr_evaluate/main.cpp:536-563, 676-690: 5e-5 of the largest bounding-box
    extent for positions, 5x for first and 25x for second derivatives."""
    p = np.asarray(positions, np.float64).reshape(-1, 3)
    ptol = 5e-5 * float((p.max(0) - p.min(0)).max())
    return (ptol, 5 * ptol, 5 * ptol, 25 * ptol, 25 * ptol, 25 * ptol)


@pytest.mark.gpu
def test_pattern_sweep_matches_the_reference():
    torch_cuda()
    from opensubdiv_gb300 import bfr
    z = np.load(os.path.join(GOLDEN, "bfr_tess_patterns.npz"))
    meta, ro, rates = z["meta"], z["rate_offsets"], z["rates"]
    groups = {}
    for i in range(len(meta)):
        reg, N, fs, pq = (int(x) for x in meta[i][:4])
        groups.setdefault((reg, fs, pq), []).append(i)
    checked = 0
    for (reg, fs, pq), idx in groups.items():
        sizes = np.array([meta[i][1] for i in idx], np.int32)
        runs = [rates[ro[i]:ro[i + 1]] for i in idx]
        r_off = np.concatenate([[0], np.cumsum([len(r) for r in runs])]).astype(np.int32)
        m = bfr.MeshTessellation(reg, sizes, rates=np.concatenate(runs), rate_offsets=r_off,
                                 options=bfr.TessellationOptions(fs, pq))
        c, f, _ = m.Generate(offset_facet_indices=False)
        c, f = host(c), host(f)
        co, fo = host(m.coord_offsets), host(m.facet_offsets)
        for j, i in enumerate(idx):
            want_c = z["coords"][z["coord_offsets"][i]:z["coord_offsets"][i + 1]]
            want_f = z["facets"][z["facet_offsets"][i]:z["facet_offsets"][i + 1]]
            assert co[j + 1] - co[j] == len(want_c), i
            assert (fo[j + 1] - fo[j]) * f.shape[1] == len(want_f), i
            assert np.array_equal(bits(c[co[j]:co[j + 1]]), bits(want_c)), i
            assert np.array_equal(f[fo[j]:fo[j + 1]].ravel(), want_f), i
            checked += 1
    assert checked == len(meta)


@pytest.mark.gpu
@pytest.mark.parametrize("reg,fs,pq", [(4, 3, 0), (4, 4, 0), (4, 4, 1), (3, 3, 0), (3, 4, 1)])
def test_uniform_rate_patterns_and_mesh_offsets(reg, fs, pq):
    """A single uniform rate (faces of 3..10 sides share one device pattern each, larger
    polygons are generated per face), mesh-wide facet indices and ptex offsets."""
    torch_cuda()
    from opensubdiv_gb300 import bfr
    rng = np.random.default_rng(reg * 10 + fs + pq)
    pool = [3, 4, 5, 6, 7, 8, 9, 10, 11, 13] if reg == 4 else [3, 3, 3, 4]
    sizes = rng.choice(pool, 400).astype(np.int32)
    for rate in (1, 2, 3, 4, 5, 8, 13):
        m = bfr.MeshTessellation(reg, sizes, uniform_rate=rate,
                                 options=bfr.TessellationOptions(fs, pq))
        c, f, _ = m.Generate()
        c, f = host(c), host(f)
        co, fo, po = host(m.coord_offsets), host(m.facet_offsets), host(m.ptex_offsets)
        assert np.array_equal(np.diff(po), np.where(sizes == reg, 1, sizes))
        for j, N in enumerate(sizes):
            want = oracle.tess_generate(reg, int(N), [rate], fs, pq)
            if want is None:
                assert co[j + 1] == co[j] and fo[j + 1] == fo[j]
                continue
            wc, wf = want
            assert np.array_equal(bits(c[co[j]:co[j + 1]]), bits(wc)), (rate, j, N)
            got = f[fo[j]:fo[j + 1]]
            assert np.array_equal(np.where(got >= 0, got - co[j], -1), wf), (rate, j, N)


@pytest.mark.gpu
def test_strides_and_face_local_indices():
    """Coord and facet strides of Tessellation::Options: only the (u,v) pair and facet size
    entries of each record are written."""
    torch = torch_cuda()
    from opensubdiv_gb300 import bfr
    sizes = np.array([4, 5, 3, 4], np.int32)
    rates = np.array([3, 1, 2, 4, 5, 2, 2, 3, 2, 6, 3, 3, 1, 2, 4], np.int32)
    r_off = np.array([0, 4, 9, 12, 15], np.int32)
    opt = bfr.TessellationOptions(4, 1, coord_stride=3, facet_stride=6)
    m = bfr.MeshTessellation(4, sizes, rates=rates, rate_offsets=r_off, options=opt)
    c = torch.full((m.num_coords, 3), 7.0, device="cuda")
    f = torch.full((m.num_facets, 6), -9, dtype=torch.int32, device="cuda")
    m.Generate(coords=c, facets=f, offset_facet_indices=False)
    c, f = host(c), host(f)
    assert (c[:, 2] == 7.0).all() and (f[:, 4:] == -9).all()
    co, fo = host(m.coord_offsets), host(m.facet_offsets)
    for j in range(len(sizes)):
        wc, wf = oracle.tess_generate(4, int(sizes[j]), rates[r_off[j]:r_off[j + 1]], 4, True)
        assert np.array_equal(bits(c[co[j]:co[j + 1], :2]), bits(wc))
        assert np.array_equal(f[fo[j]:fo[j + 1], :4], wf)


@pytest.mark.gpu
def test_invalid_requests_are_rejected():
    torch_cuda()
    from opensubdiv_gb300 import bfr
    from opensubdiv_gb300._lib import GB300Error
    with pytest.raises(GB300Error):
        bfr.MeshTessellation(5, np.array([4], np.int32), uniform_rate=3)
    with pytest.raises(GB300Error):
        bfr.MeshTessellation(4, np.array([4], np.int32), uniform_rate=3,
                             options=bfr.TessellationOptions(3, 0, coord_stride=1))
    # invalid faces (rate 0, a 2-gon) tessellate to nothing, like an invalid Bfr::Tessellation
    m = bfr.MeshTessellation(4, np.array([4, 2, 5], np.int32), rates=np.array([0, 3, 2], np.int32))
    want = oracle.tess_inventory(4, 5, [2])[1]
    assert list(np.diff(host(m.coord_offsets))) == [0, 0, want]


@pytest.mark.gpu
@pytest.mark.parametrize("path", MESHES, ids=os.path.basename)
def test_mesh_tessellate_and_evaluate_matches_bfr(path):
    torch = torch_cuda()
    from opensubdiv_gb300 import bfr
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300PatchTable
    z = np.load(path)
    name = os.path.basename(path)[:-4]
    reg = int(z["regular_face_size"])
    table = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"],
                                   bool(z["triangular"]))
    opt = bfr.TessellationOptions(int(z["facet_size"]), bool(z["preserve_quads"]))
    m = bfr.MeshTessellation(reg, z["verts_per_face"], rates=z["rates"],
                             rate_offsets=z["rate_offsets"], options=opt)
    assert np.array_equal(host(m.coord_offsets), z["coord_offsets"])
    assert np.array_equal(host(m.ptex_offsets), z["ptex_offsets"])
    c, f, pc = m.Generate(table=table)
    assert np.array_equal(bits(host(c)), bits(z["coords"]))
    assert np.array_equal(host(f), z["facets"])
    pc = host(pc)
    assert np.array_equal(pc[:, :3], z["q_handles"])
    assert np.array_equal(pc[:, 3], bits(z["q_s"]))
    assert np.array_equal(pc[:, 4], bits(z["q_t"]))
    outs = [host(o) for o in m.Evaluate(dev(z["src"]), BD(0, 3, 3), table, dev(pc), 2)]
    tol = bfr_tolerances(z["positions"])
    n = m.num_coords
    cpu = [np.zeros(n * 3, np.float32) for _ in range(6)]
    f64 = [np.zeros(n * 3) for _ in range(6)]
    tab = (pc, z["arrays"], z["patch_indices"], z["params"])
    assert oracle.eval_patches(z["src"], (0, 3, 3), cpu, [(0, 3, 3)] * 6, *tab, threads=4)
    assert oracle.eval_patches(z["src"], (0, 3, 3), f64, [(0, 3, 3)] * 6, *tab, threads=4,
                               fp64=True)
    diag = bbox_diag(z["positions"])
    from test_bfr_oracle import rotated_triangles, second_derivative_error
    rot = rotated_triangles(z)
    for k in range(6):
        got = outs[k].astype(np.float64)
        err = np.abs(got - z["out6"][k])
        if k >= 3:  # Far's sign on rotated triangle sub-patches (tests/test_bfr_oracle.py)
            err = np.minimum(err, second_derivative_error(got, z["out6"][k], rot))
        assert err.max() <= tol[k], (name, k, err.max(), tol[k])
        gate(f"bfr {name}", k, outs[k].ravel(), cpu[k], f64[k], diag)


@pytest.mark.gpu
@pytest.mark.parametrize("reg,fs,pq,offset,strides", [(4, 3, 0, True, (0, 0)),
                                                      (4, 4, 1, False, (3, 6)),
                                                      (3, 4, 0, True, (0, 5))])
def test_per_face_rates_with_repeated_tuples(reg, fs, pq, offset, strides):
    """Per-face rate runs drawn from a small set, so most faces share their (size, rates) with
    others: one face per tuple generates the pattern, the rest copy it from that face's output
    slice (indices moved to their own coords).  Every face against the oracle."""
    torch = torch_cuda()
    from opensubdiv_gb300 import bfr
    rng = np.random.default_rng(77 + reg + fs)
    nfaces = 3000
    pool = [3, 4, 4, 4, 5, 6, 11] if reg == 4 else [3, 3, 3, 4]
    sizes = rng.choice(pool, nfaces).astype(np.int32)
    runs = []
    for N in sizes:
        kind = rng.integers(0, 3)
        if kind == 0:
            runs.append(rng.integers(1, 4, 1))
        elif kind == 1:
            runs.append(rng.integers(2, 5, N))
        else:
            runs.append(rng.integers(2, 4, N + 1))
    r_off = np.concatenate([[0], np.cumsum([len(r) for r in runs])]).astype(np.int32)
    rates = np.concatenate(runs).astype(np.int32)
    cs, fst = strides
    opt = bfr.TessellationOptions(fs, pq, coord_stride=cs, facet_stride=fst)
    m = bfr.MeshTessellation(reg, sizes, rates=rates, rate_offsets=r_off, options=opt)
    c, f, _ = m.Generate(offset_facet_indices=offset)
    c, f = host(c), host(f)
    co, fo = host(m.coord_offsets), host(m.facet_offsets)
    for j in range(nfaces):
        want = oracle.tess_generate(reg, int(sizes[j]), rates[r_off[j]:r_off[j + 1]], fs, pq)
        if want is None:
            assert co[j + 1] == co[j]
            continue
        wc, wf = want
        assert np.array_equal(bits(c[co[j]:co[j + 1], :2]), bits(wc)), j
        got = f[fo[j]:fo[j + 1], :wf.shape[1]]
        if offset:
            got = np.where(got >= 0, got - co[j], -1)
        assert np.array_equal(got, wf), j


UV_MESHES = [p for p in MESHES if "_uv_" in os.path.basename(p)]


@pytest.mark.gpu
@pytest.mark.parametrize("path", UV_MESHES, ids=os.path.basename)
def test_mesh_face_varying_uvs_match_bfr(path):
    """The reference's tutorial 1.3: UVs of every tessellation coord from the face-varying
    surfaces.  On the device: the tessellation's PatchCoords (vertex PatchMap) evaluated on the
    table's face-varying channel (EvaluateFaceVarying), against Bfr within the reference's UV
    tolerance, and against the oracle's evaluation of the same face-varying patches."""
    torch = torch_cuda()
    from opensubdiv_gb300 import bfr
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300PatchTable
    z = np.load(path)
    reg = int(z["regular_face_size"])
    table = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"],
                                   bool(z["triangular"]))
    ch = table.AddFVarChannel(z["fvar_arrays"], z["fvar_indices"], z["fvar_params"])
    opt = bfr.TessellationOptions(int(z["facet_size"]), bool(z["preserve_quads"]))
    m = bfr.MeshTessellation(reg, z["verts_per_face"], rates=z["rates"],
                             rate_offsets=z["rate_offsets"], options=opt)
    c, f, pc = m.Generate(table=table)
    outs = [host(o) for o in m.EvaluateFaceVarying(dev(z["fvar_src"]), BD(0, 2, 2), table, pc,
                                                   ch, 1)]
    n = m.num_coords
    cpu = [np.zeros(n * 2, np.float32) for _ in range(3)]
    assert oracle.eval_patches(z["fvar_src"], (0, 2, 2), cpu, [(0, 2, 2)] * 3, host(pc),
                               z["fvar_arrays"], z["fvar_indices"], z["fvar_params"], threads=4)
    for k, tol in enumerate((1e-4, 5e-4, 5e-4)):
        assert np.abs(outs[k] - z["uv3"][k]).max() <= tol, k
        assert np.abs(outs[k].ravel() - cpu[k]).max() <= 1e-5, k


SHARE = os.path.join(GOLDEN, "bfr_share.npz")


@pytest.mark.gpu
@pytest.mark.parametrize("path", MESHES, ids=os.path.basename)
@pytest.mark.parametrize("local", [False, True], ids=["mesh", "local"])
def test_mesh_shared_points_match_the_reference_tutorial(path, local):
    """Shared (watertight) points on the device (GB300TessellationShare) against the
    reference's tutorial 2.2 loop (tests/golden/bfr_share.npz): facets as point indices and
    each face's first point exactly; each point's PatchCoord, (u, v) and face copied from the
    coord that made it; vertex and edge points as the oracle's bookkeeping numbers them; and
    the points evaluated once each equal the per-coord evaluation bit for bit."""
    torch = torch_cuda()
    from opensubdiv_gb300 import bfr
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300PatchTable
    z = np.load(path)
    g = np.load(SHARE)
    key = os.path.basename(path)[:-4]
    reg = int(z["regular_face_size"])
    table = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"],
                                   bool(z["triangular"]))
    opt = bfr.TessellationOptions(int(z["facet_size"]), bool(z["preserve_quads"]))
    m = bfr.MeshTessellation(reg, z["verts_per_face"], rates=z["rates"],
                             rate_offsets=z["rate_offsets"], options=opt)
    c, f, pc = m.Generate(table=table, offset_facet_indices=not local)
    fe, ne = oracle.edge_numbering(z["verts_per_face"], z["face_verts"])
    nv = len(z["positions"])
    coord_facets = host(f).copy()
    sp = m.Share(z["face_verts"], fe, nv, ne, f, patch_coords=pc, coords=c,
                 mesh_facet_indices=not local, point_coords=True, point_faces=True,
                 vertex_points=True, edge_points=True)
    src = g[key + "__point_sources"]
    assert sp.num_points == len(src)
    assert np.array_equal(host(f), g[key + "__facets"])
    assert np.array_equal(host(sp.point_offsets), g[key + "__point_offsets"])
    assert np.array_equal(host(sp.patch_coords), host(pc)[src])
    assert np.array_equal(bits(host(sp.coords)), bits(host(c)[src]))
    co = z["coord_offsets"]
    assert np.array_equal(host(sp.faces), np.searchsorted(co, src, side="right") - 1)
    # vertex points: the point every face corner's vertex coord maps to
    fs = int(z["facet_size"])
    cf = coord_facets.reshape(-1, fs)
    pf = host(f).reshape(-1, fs)
    if local:
        fo = z["facet_offsets"]
        owner = np.repeat(np.arange(len(co) - 1), np.diff(fo))
        cf = np.where(cf >= 0, cf + co[owner][:, None], -1)
    point_of_coord = np.full(int(co[-1]), -1, np.int64)
    point_of_coord[cf[cf >= 0]] = pf[cf >= 0]
    vp = host(sp.vertex_points)
    starts = np.concatenate([[0], np.cumsum(z["verts_per_face"])])
    for fi in range(len(co) - 1):
        if co[fi + 1] == co[fi]:
            continue
        r = z["rates"][z["rate_offsets"][fi]:z["rate_offsets"][fi + 1]]
        N = int(z["verts_per_face"][fi])
        outer = np.broadcast_to(r[:N] if len(r) >= N else r[:1], (N,))
        pos = co[fi] + np.concatenate([[0], np.cumsum(outer)[:-1]])
        verts = z["face_verts"][starts[fi]:starts[fi + 1]]
        assert np.array_equal(vp[verts], point_of_coord[pos]), fi
    # evaluate each point once: equal to the evaluation at the coord that made it
    per_coord = [host(o) for o in m.Evaluate(dev(z["src"]), BD(0, 3, 3), table, pc, 1)]
    per_point = [host(o) for o in m.Evaluate(dev(z["src"]), BD(0, 3, 3), table,
                                             sp.patch_coords, 1, num_points=sp.num_points)]
    for k in range(3):
        assert np.array_equal(bits(per_point[k]), bits(per_coord[k][src])), k


@pytest.mark.gpu
def test_shared_points_reject_bad_edges():
    """Two rates on one shared edge, and vertex or edge indices out of range, are rejected
    (the device checks every index before it uses it)."""
    torch_cuda()
    from opensubdiv_gb300 import bfr
    from opensubdiv_gb300._lib import GB300Error
    sizes = np.array([4, 4], np.int32)
    fv = np.array([0, 1, 4, 3, 1, 2, 5, 4], np.int32)
    fe, ne = oracle.edge_numbering(sizes, fv)
    ro = np.array([0, 4, 8], np.int32)
    for rates, verts, edges, nedges in (
            ([2, 3, 2, 3, 2, 3, 2, 4], fv, fe, ne),  # two rates on the shared edge
            ([2, 3, 2, 3, 2, 3, 2, 3], fv, fe, ne - 1),  # an edge index out of range
            ([2, 3, 2, 3, 2, 3, 2, 3], np.where(fv == 5, 6, fv), fe, ne),  # a vertex index
            ([2, 3, 2, 3, 2, 3, 2, 3], fv[:-1], fe[:-1], ne)):  # fewer corners than sizes
        m = bfr.MeshTessellation(4, sizes, rates=np.array(rates, np.int32), rate_offsets=ro)
        _, f, _ = m.Generate()
        with pytest.raises(GB300Error):
            m.Share(verts, edges, 6, nedges, f)
    # the consistent mesh shares the edge: 6 vertices + 4 * 2 + 3 * 1 edge points + interior
    m = bfr.MeshTessellation(4, sizes, rates=np.array([2, 3, 2, 3] * 2, np.int32),
                             rate_offsets=ro)
    _, f, _ = m.Generate()
    sp = m.Share(fv, fe, 6, ne, f)
    mesh = oracle.tess_mesh(4, sizes, ro, np.array([2, 3, 2, 3] * 2, np.int32))
    want, po, src = oracle.tess_share(4, sizes, fv, fe, 6, ne, ro, np.array([2, 3, 2, 3] * 2),
                                      mesh["coord_offsets"], mesh["facet_offsets"],
                                      mesh["facets"])
    assert sp.num_points == len(src)
    assert np.array_equal(host(f), want)


@pytest.mark.gpu
@pytest.mark.parametrize("key", STENCIL_MESHES)
def test_point_stencils_on_the_device(key):
    """GB300TessellationStencils (Bfr::Surface::EvaluateStencil at every coord): the device
    masks merged over the patch points' stencils hold the same entries as the oracle's merge
    (rows compared with sorted entries) with weights within float rounding; evaluated from the
    cage by EvalStencils they give GB300TessellationEvaluate's points (flat 1e-5 x bbox
    diagonal) and Bfr::Surface::Evaluate's within the reference's Bfr-versus-Far tolerances."""
    torch = torch_cuda()
    from opensubdiv_gb300 import bfr
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300PatchTable, GB300StencilTable)
    z = np.load(os.path.join(GOLDEN, key + ".npz"))
    g = np.load(STENCILS)
    table = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"],
                                   bool(z["triangular"]))
    opt = bfr.TessellationOptions(int(z["facet_size"]), bool(z["preserve_quads"]))
    m = bfr.MeshTessellation(int(z["regular_face_size"]), z["verts_per_face"], rates=z["rates"],
                             rate_offsets=z["rate_offsets"], options=opt)
    _, _, pc = m.Generate(table=table)
    bh = point_base(z, g, key)
    base = GB300StencilTable.Create(bh["sizes"], bh["offsets"], bh["indices"], bh["weights"])
    st = GB300StencilTable.FromPatchCoords(table, pc, base, channels=3)
    h = st.CopyToHost()
    want = oracle_point_stencils(z, bh)
    assert np.array_equal(h["sizes"], want["sizes"])
    o = np.concatenate([[0], np.cumsum(want["sizes"])])
    for name in ("weights", "du_weights", "dv_weights"):
        scale = max(1.0, float(np.abs(want[name]).max()))
        for i in range(len(want["sizes"])):
            a, b = slice(h["offsets"][i], h["offsets"][i] + h["sizes"][i]), slice(o[i], o[i + 1])
            pa, pb = np.argsort(h["indices"][a]), np.argsort(want["indices"][b])
            assert np.array_equal(h["indices"][a][pa], want["indices"][b][pb]), (key, i)
            err = np.abs(h[name][a][pa] - want[name][b][pb]).max()
            assert err <= 4e-6 * scale, (key, name, i, err, scale)
    n = m.num_coords
    d = BD(0, 3, 3)
    outs = [torch.zeros(n * 3, device="cuda") for _ in range(3)]
    assert Ev.EvalStencilsTable(dev(z["positions"].ravel()), d, outs[0], d, st, du=outs[1],
                                duDesc=d, dv=outs[2], dvDesc=d)
    per = m.Evaluate(dev(z["src"]), d, table, pc, 1)
    diag = bbox_diag(z["positions"])
    tol = bfr_tolerances(z["positions"])
    for k in range(3):
        got = host(outs[k]).reshape(-1, 3).astype(np.float64)
        assert np.abs(got - host(per[k]).reshape(-1, 3)).max() <= 1e-5 * diag * (1 if k == 0 else 4), k
        assert np.abs(got - z["out6"][k]).max() <= tol[k], k


@pytest.mark.gpu
@pytest.mark.parametrize("key", STENCIL_MESHES)
def test_mesh_varying_values_match_bfr(key):
    """Varying surfaces (InitVaryingSurface) at every coord on the device: the values refined
    by EvalStencils with Far's varying stencils, then MeshTessellation.EvaluateVarying at the
    located coords -- within 1e-6 of the reference's Bfr varying evaluation."""
    torch = torch_cuda()
    from opensubdiv_gb300 import bfr
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300PatchTable, GB300StencilTable)
    z = np.load(os.path.join(GOLDEN, key + ".npz"))
    g = np.load(STENCILS)
    table = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"],
                                   bool(z["triangular"]))
    table.SetVarying(g[f"{key}__var_arrays"], g[f"{key}__var_indices"])
    opt = bfr.TessellationOptions(int(z["facet_size"]), bool(z["preserve_quads"]))
    m = bfr.MeshTessellation(int(z["regular_face_size"]), z["verts_per_face"], rates=z["rates"],
                             rate_offsets=z["rate_offsets"], options=opt)
    _, _, pc = m.Generate(table=table)
    vals = g[f"{key}__var_values"]
    nc = len(vals)
    vst = GB300StencilTable.Create(g[f"{key}__var_st_sizes"], g[f"{key}__var_st_offsets"],
                                   g[f"{key}__var_st_indices"], g[f"{key}__var_st_weights"])
    src = torch.zeros((nc + vst.GetNumStencils()) * 3, device="cuda")
    src[: nc * 3] = dev(vals.ravel())
    assert Ev.EvalStencilsTable(src, BD(0, 3, 3), src, BD(nc * 3, 3, 3), vst)
    (val,) = m.EvaluateVarying(src, BD(0, 3, 3), table, pc)
    assert np.abs(host(val) - g[f"{key}__var_bfr"]).max() <= 1e-6


def tutorial_rates(points_per_corner, sizes, interval, max_rate):
    """Tutorial 2.1's rule on host points, one per face corner (float arithmetic)."""
    sizes = np.asarray(sizes, np.int64)
    start = np.concatenate([[0], np.cumsum(sizes)])
    nxt = np.arange(start[-1]) + 1
    nxt[start[1:] - 1] = start[:-1]
    p = np.asarray(points_per_corner, np.float32).reshape(-1, 3)
    dv = np.abs(p - p[nxt])
    length = np.sqrt(dv[:, 0] * dv[:, 0] + dv[:, 1] * dv[:, 1] + dv[:, 2] * dv[:, 2])
    return np.minimum(1 + (length / np.float32(interval)).astype(np.int32), max_rate)


@pytest.mark.gpu
@pytest.mark.parametrize("path", MESHES[:4] + [os.path.join(GOLDEN, "large", "torus512x256_bfr.npz")],
                         ids=os.path.basename)
def test_edge_rates_follow_tutorial_2_1(path):
    """GB300TessellationEdgeRates: with the control hull (mesh-vertex points) the rates equal
    tutorial 2.1's rule computed on the host bit for bit, shared edges get one rate from both
    faces, and the offsets are the face sizes' scan; with limit points (one per face corner:
    the limit surface evaluated at the rate-1 tessellation's vertex coords, the tutorial's
    other option) they equal the rule on the same points."""
    if not os.path.exists(path):
        pytest.skip("large fixture is written where the reference is available")
    torch_cuda()
    from opensubdiv_gb300 import bfr, workloads
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300PatchTable
    z = np.load(path)
    sizes, fv, pos = z["verts_per_face"], z["face_verts"], z["positions"]
    ext = float((pos.max(0) - pos.min(0)).max())
    interval, max_rate = ext / 40.0, 10
    off, rates = bfr.EdgeRates(sizes, fv, pos, interval, max_rate)
    want_off, want = workloads.bfr_edge_length_rates(pos, sizes, fv, interval, max_rate)
    assert np.array_equal(host(off), want_off)
    assert np.array_equal(host(rates), want)
    assert np.array_equal(want, tutorial_rates(pos[fv], sizes, interval, max_rate))
    fe, ne = workloads.face_edges(sizes, fv)
    per_edge = np.full(ne, -1)
    per_edge[fe] = want
    assert np.array_equal(per_edge[fe], want)
    # limit option: points at the faces' corners on the limit surface
    reg = int(z["regular_face_size"]) if "regular_face_size" in z.files else 4
    tri = bool(z["triangular"])
    table = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"], tri)
    m = bfr.MeshTessellation(reg, sizes, uniform_rate=1)
    _, _, pc = m.Generate(table=table)
    co = host(m.coord_offsets)
    (P,) = m.Evaluate(dev(z["src"]), BD(0, 3, 3), table, pc, 0)
    P = host(P)
    valid = np.diff(co) > 0
    corners = np.concatenate([np.arange(co[f], co[f] + sizes[f]) for f in np.nonzero(valid)[0]])
    vs = sizes[valid]
    cp = np.ascontiguousarray(P[corners], np.float32)
    _, lrates = bfr.EdgeRates(vs, np.zeros(int(vs.sum()), np.int32), cp, interval, max_rate,
                              points_per_corner=True)
    assert np.array_equal(host(lrates), tutorial_rates(cp, vs, interval, max_rate))


@pytest.mark.gpu
def test_edge_rates_reject_bad_topology():
    torch_cuda()
    from opensubdiv_gb300 import bfr
    from opensubdiv_gb300._lib import GB300Error
    pos = np.zeros((6, 3), np.float32)
    with pytest.raises(GB300Error):
        bfr.EdgeRates(np.array([4, 4], np.int32), np.array([0, 1, 4, 3, 1, 2, 5], np.int32),
                      pos, 0.1)
    with pytest.raises(GB300Error):
        bfr.EdgeRates(np.array([4, 4], np.int32), np.array([0, 1, 4, 3, 1, 2, 9, 4], np.int32),
                      pos, 0.1)
