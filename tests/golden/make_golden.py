"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a container that has the reference sources (it builds oracle/_ref/libosdref.so, the
reference's own Far + Osd CPU code compiled from source, and drives it through
oracle/ref_shim.cpp):

    make -C oracle ref && python tests/golden/make_golden.py [mode]

Modes: none (the stencil and patch fixtures), `regression`, `factory`, `bfr` (the Bfr pattern
sweep, the mesh fixtures, shared points and limit stencils), `bfr-share`, `bfr-stencils`, and
`large`, `bfr-large`, `bfr-stencils-large` (full-size workloads under large/, kept out of git).

Every array written here comes out of the reference: Far factories build the tables,
Osd::CpuEvaluator produces the float outputs, Far::PatchMap the handles,
Far::PatchTable::EvaluateBasis<double> the FP64 outputs, and Bfr (SurfaceFactory, Surface,
Tessellation) the Bfr outputs, through the reference tutorials' loops.  The cages are the
seeded synthetic shapes of opensubdiv_gb300/shapes.py at reduced sizes.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from opensubdiv_gb300 import shapes  # noqa: E402
import ref  # noqa: E402


def cage_arrays(cage):
    return dict(positions=cage.positions, verts_per_face=cage.verts_per_face,
                face_verts=cage.face_verts, scheme=np.int32(cage.scheme),
                crease_verts=np.asarray(cage.crease_verts, np.int32).reshape(-1, 2),
                crease_sharpness=np.asarray(cage.crease_sharpness, np.float32))


def eval_cpu(src, sdesc, table, nout, ddescs, n_dst, dst_len):
    outs = [np.zeros(n_dst, np.float32) for _ in range(nout)]
    names = ("du", "dv", "duu", "duv", "dvv")[: nout - 1]
    ws = [table["weights"]] + [table[k + "_weights"] for k in names]
    ok = ref.cpu_eval_stencils(src, sdesc, outs, ddescs, table["sizes"], table["offsets"],
                               table["indices"], ws, 0, len(table["sizes"]))
    assert ok
    return outs


def stencil_fixture(path, cage, level, seed, limit_level=None, nlimit=0):
    rng = np.random.default_rng(seed)
    out = dict(cage_arrays(cage))
    r = ref.Refiner(cage).refine_uniform(level)
    st = ref.stencil_table(r, intermediate=False)
    std = ref.stencil_table(r, use_double=True, intermediate=False)
    assert np.array_equal(st["indices"], std["indices"])
    n = len(st["sizes"])
    nc = cage.num_vertices
    out.update(level=np.int32(level), sizes=st["sizes"], offsets=st["offsets"],
               indices=st["indices"], weights=st["weights"], weights_fp64=std["weights"])
    # xyz, stride 3
    src3 = cage.positions.reshape(-1).copy()
    out["out3"] = eval_cpu(src3, (0, 3, 3), st, 1, [(0, 3, 3)], n * 3, 3)[0]
    # 8 interleaved primvars: xyz + 5 channels U[-1, 1]
    src8 = np.concatenate([cage.positions, rng.uniform(-1, 1, (nc, 5)).astype(np.float32)], 1)
    src8 = src8.astype(np.float32).reshape(-1)
    out["src8"] = src8
    out["out8"] = eval_cpu(src8, (0, 8, 8), st, 1, [(0, 8, 8)], n * 8, 8)[0]
    # strided + offset descriptors: source stride 7 (xyz at 2), destination stride 5 (at 1)
    src7 = rng.uniform(-1, 1, (nc, 7)).astype(np.float32)
    src7[:, 2:5] = cage.positions
    src7 = src7.reshape(-1)
    out["src7"] = src7
    out["out_strided"] = eval_cpu(src7, (2, 3, 7), st, 1, [(1, 3, 5)], n * 5 + 5, 3)[0]
    # in place, the way Osd::Mesh::Refine calls it (osd/mesh.h:501-540)
    buf = np.zeros((nc + n) * 3, np.float32)
    buf[: nc * 3] = cage.positions.reshape(-1)
    ok = ref.cpu_eval_stencils(buf, (0, 3, 3), [buf], [(nc * 3, 3, 3)], st["sizes"],
                               st["offsets"], st["indices"], [st["weights"]], 0, n)
    assert ok
    out["out_inplace"] = buf
    if limit_level is not None and nlimit > 0:
        ra = ref.Refiner(cage).refine_adaptive(limit_level)
        face, u, v = shapes.uniform_locations(cage, nlimit, seed=seed + 7)
        lt = ref.limit_stencil_table(ra, face, u, v, d1=True, d2=True)
        ltd = ref.limit_stencil_table(ra, face, u, v, use_double=True, d1=True, d2=True)
        assert np.array_equal(lt["indices"], ltd["indices"])
        m = len(lt["sizes"])
        out.update(limit_level=np.int32(limit_level), limit_face=face, limit_u=u, limit_v=v)
        for k in ("sizes", "offsets", "indices", "weights", "du_weights", "dv_weights",
                  "duu_weights", "duv_weights", "dvv_weights"):
            out["limit_" + k] = lt[k]
            if k.endswith("weights"):
                out["limit_" + k + "_fp64"] = ltd[k]
        o6 = eval_cpu(src3, (0, 3, 3), lt, 6, [(0, 3, 3)] * 6, m * 3, 3)
        o3 = eval_cpu(src3, (0, 3, 3), lt, 3, [(0, 3, 3)] * 3, m * 3, 3)
        for a, b in zip(o3, o6[:3]):
            assert np.array_equal(a, b)
        out["limit_out6"] = np.stack(o6)
    np.savez_compressed(path, **out)
    return out


def edge_queries(nptex, rng, n):
    """Queries on exact quadrant medians, corners and the largest float below 1."""
    vals = np.array([0.0, 0.5, 1.0, 0.25, 0.75, 0.125, 0.375, np.nextafter(np.float32(1), 0),
                     0.0625, 0.9375], np.float32)
    face = rng.integers(0, nptex, n).astype(np.int32)
    u = vals[rng.integers(0, len(vals), n)]
    v = vals[rng.integers(0, len(vals), n)]
    return face, u, v


def uv_seams(cage, nu, nv):
    """A face-varying UV channel with seams for a shapes.torus(nu, nv) cage: values on an
    (nu + 1) x (nv + 1) grid, so faces across the wrap use the duplicated seam values.
    Returns (number of values, value index per face-vertex)."""
    fidx = []
    start = 0
    for n in cage.verts_per_face:
        vs = cage.face_verts[start:start + n]
        start += n
        i, j = vs // nv, vs % nv
        if i.max() - i.min() > 1:
            i = np.where(i == 0, nu, i)
        if j.max() - j.min() > 1:
            j = np.where(j == 0, nv, j)
        fidx.extend((i * (nv + 1) + j).tolist())
    return (nu + 1) * (nv + 1), np.asarray(fidx, np.int32)


def uv_grid(nu, nv):
    """The texture coordinates of uv_seams' values: value i * (nv + 1) + j = (i / nu, j / nv)."""
    i, j = np.meshgrid(np.arange(nu + 1), np.arange(nv + 1), indexing="ij")
    return np.stack([i.ravel() / nu, j.ravel() / nv], 1).astype(np.float32)


def patch_fixture(path, cage, level, seed, nq=3000, adaptive=True, endcap=3, fvar=None):
    """fvar: (num_values, indices per face-vertex) of a face-varying channel; the fixture then
    also holds the reference's varying and face-varying patch tables with CpuEvaluator
    outputs over random sources (EvalPatchesVarying / EvalPatchesFaceVarying)."""
    rng = np.random.default_rng(seed)
    out = dict(cage_arrays(cage))
    r = ref.Refiner(cage, fvar=None if fvar is None else (fvar[0], fvar[1], False))
    if adaptive:
        r.refine_adaptive(level)
    else:
        r.refine_uniform(level)
    p = ref.Patches(r, endcap=endcap, max_isolation=level)
    nc = cage.num_vertices
    ns = len(p.st["sizes"])
    buf = np.zeros((nc + ns) * 3, np.float32)
    buf[: nc * 3] = cage.positions.reshape(-1)
    ok = ref.cpu_eval_stencils(buf, (0, 3, 3), [buf], [(nc * 3, 3, 3)], p.st["sizes"],
                               p.st["offsets"], p.st["indices"], [p.st["weights"]], 0, ns)
    assert ok
    nptex = r.num_ptex_faces()
    f1, u1, v1 = shapes.uniform_locations(cage, nq, seed=seed + 3)
    f2, u2, v2 = edge_queries(nptex, rng, nq // 10)
    # out-of-range faces: FindPatch returns NULL (far/patchMap.h:205)
    f3 = np.array([-1, nptex, nptex + 5], np.int32)
    u3 = np.array([0.5, 0.5, 0.1], np.float32)
    v3 = np.array([0.5, 0.2, 0.1], np.float32)
    faces = np.concatenate([f1, f2, f3])
    u = np.concatenate([u1, u2, u3])
    v = np.concatenate([v1, v2, v3])
    if cage.scheme == shapes.LOOP:
        fold = (u + v) > 1.0
        u[fold] = 1.0 - u[fold]
        v[fold] = 1.0 - v[fold]
    handles, found = p.find_patches(faces, u.astype(np.float64), v.astype(np.float64))
    sel = np.nonzero(found)[0]
    coords = np.zeros((len(sel), 5), np.int32)
    coords[:, :3] = handles[sel]
    coords[:, 3] = u[sel].view(np.int32)
    coords[:, 4] = v[sel].view(np.int32)
    outs = [np.zeros(len(sel) * 3, np.float32) for _ in range(6)]
    ok = ref.cpu_eval_patches(buf, (0, 3, 3), outs, [(0, 3, 3)] * 6, coords, p.arrays,
                              p.indices, p.params)
    assert ok
    fp64 = p.eval_fp64(buf, 3, 3, handles[sel], u[sel].astype(np.float64),
                       v[sel].astype(np.float64))
    out.update(level=np.int32(level), adaptive=np.int32(adaptive), endcap=np.int32(endcap),
               arrays=p.arrays, patch_indices=p.indices, params=p.params,
               num_local_points=np.int32(p.num_local_points), src=buf,
               # the patch points' stencils over the cage (all refinement levels + local
               # points): src[nc:] = these stencils applied to src[:nc]
               ps_sizes=p.st["sizes"], ps_offsets=p.st["offsets"], ps_indices=p.st["indices"],
               ps_weights=p.st["weights"],
               num_ptex=np.int32(nptex), q_face=faces, q_u=u, q_v=v, q_handles=handles,
               q_found=found, coords=coords, out6=np.stack(outs).reshape(6, -1, 3),
               out6_fp64=fp64.transpose(1, 0, 2).copy(),
               triangular=np.int32(cage.scheme == shapes.LOOP))
    if fvar is not None:
        # varying: the vertex patch params with the varying arrays / indices, 4 primvars
        va, vi = p.varying()
        vsrc = rng.uniform(-1, 1, (int(vi.max()) + 1, 4)).astype(np.float32).ravel()
        vouts = [np.zeros(len(sel) * 4, np.float32) for _ in range(3)]
        assert ref.cpu_eval_patches(vsrc, (0, 4, 4), vouts, [(0, 4, 4)] * 3, coords, va, vi,
                                    p.params)
        # face-varying channel 0: its own arrays / indices / params, 2 primvars (uv).  The
        # source holds the channel's base values (a uv layout with seams), then its refined
        # and local-point values (Far's face-varying stencils applied by CpuEvaluator).
        fa, fi, fp = p.fvar(0)
        fst = p.fvar_stencils(r, 0)
        nbase = int(fvar[0])
        fsrc = np.zeros((nbase + len(fst["sizes"])) * 2, np.float32)
        fsrc[: nbase * 2] = fvar[2].ravel()
        assert ref.cpu_eval_stencils(fsrc, (0, 2, 2), [fsrc], [(nbase * 2, 2, 2)],
                                     fst["sizes"], fst["offsets"], fst["indices"],
                                     [fst["weights"]], 0, len(fst["sizes"]))
        assert int(fi.max()) < nbase + len(fst["sizes"])
        fouts = [np.zeros(len(sel) * 2, np.float32) for _ in range(6)]
        assert ref.cpu_eval_patches(fsrc, (0, 2, 2), fouts, [(0, 2, 2)] * 6, coords, fa, fi, fp)
        out.update(fvar_num_values=np.int32(fvar[0]), fvar_value_indices=fvar[1],
                   varying_arrays=va, varying_indices=vi, varying_src=vsrc,
                   varying_out3=np.stack(vouts).reshape(3, -1, 4),
                   fvar_arrays=fa, fvar_indices=fi, fvar_params=fp, fvar_src=fsrc,
                   fvar_out6=np.stack(fouts).reshape(6, -1, 2))
    np.savez_compressed(path, **out)
    return out


def factory_fixture(path):
    """Per-level masks recorded from Far::PrimvarRefiner (by the product's GB300MaskRecorder)
    and the tables Far::StencilTableFactory builds from the same refiners: the inputs and the
    expected outputs of the GPU stencil-table factory."""
    out = {}
    ftor = shapes.torus(12, 8, tri_fraction=0.1, crease_fraction=0.05, seed=31, noise=0.01)
    cases = [
        ("cube", shapes.cube(4, noise=0.01, seed=41), 3, ref.INTERPOLATE_VERTEX, None),
        ("torus", shapes.torus(12, 8, tri_fraction=0.1, crease_fraction=0.05, seed=42), 3,
         ref.INTERPOLATE_VERTEX, None),
        ("loop", shapes.torus(12, 8, crease_fraction=0.05, seed=43, scheme=shapes.LOOP), 3,
         ref.INTERPOLATE_VERTEX, None),
        ("varying", shapes.torus(12, 8, tri_fraction=0.1, seed=44), 2,
         ref.INTERPOLATE_VARYING, None),
        ("fvar", ftor, 2, ref.INTERPOLATE_FACE_VARYING, uv_seams(ftor, 12, 8)),
        ("pole", shapes.bipyramid(300), 1, ref.INTERPOLATE_VERTEX, None),
        ("looppole", shapes.bipyramid(300, scheme=shapes.LOOP), 1, ref.INTERPOLATE_VERTEX,
         None),
    ]
    names = []
    for name, cage, level, mode, fvar in cases:
        r = ref.Refiner(cage, fvar=None if fvar is None else (fvar[0], fvar[1], False))
        r.refine_uniform(level)
        nc, levels = ref.record_masks(r, mode)
        out[f"{name}_num_control"] = np.int32(nc)
        out[f"{name}_mode"] = np.int32(mode)
        out[f"{name}_mask_rows"] = np.array([len(d["offsets"]) - 1 for d in levels], np.int32)
        for k in ("offsets", "sources", "weights"):
            out[f"{name}_mask_{k}"] = np.concatenate([d[k] for d in levels])
        for tag, inter, ctrl in (("all", True, False), ("last_ctrl", False, True)):
            t = ref.stencil_table_mode(r, mode, intermediate=inter, control=ctrl)
            for k in ("sizes", "offsets", "indices", "weights"):
                out[f"{name}_{tag}_{k}"] = t[k]
        names.append(name)
    out["cases"] = np.array(names)
    np.savez_compressed(path, **out)


def factory_limit_fixture(path):
    """GPU LimitStencilTableFactory inputs recorded with GB300LimitStencilTableFactory's helpers
    (refined-vertex level masks, local-point masks, per-location patch points and basis
    weights from Far's own PatchMap and EvaluateBasis) and Far::LimitStencilTableFactory's
    table for the same locations."""
    out = {}
    tor = shapes.torus(12, 8, tri_fraction=0.1, crease_fraction=0.05, seed=45)
    ftor = shapes.torus(12, 8, tri_fraction=0.1, crease_fraction=0.05, seed=31, noise=0.01)
    seams = uv_seams(ftor, 12, 8)
    cases = [("adaptive", tor, 3, True, True, False, ref.INTERPOLATE_VERTEX, None),
             ("adaptive2nd", tor, 3, True, True, True, ref.INTERPOLATE_VERTEX, None),
             ("uniform", tor, 2, False, False, False, ref.INTERPOLATE_VERTEX, None),
             ("loop", shapes.icosphere(1, seed=46), 3, True, True, False,
              ref.INTERPOLATE_VERTEX, None),
             ("varying", shapes.cube(3, seed=47), 3, True, True, False,
              ref.INTERPOLATE_VARYING, None),
             ("fvar", ftor, 3, True, True, False, ref.INTERPOLATE_FACE_VARYING, seams)]
    for name, cage, level, adaptive, d1, d2, mode, fvar in cases:
        r = ref.Refiner(cage, fvar=None if fvar is None else (fvar[0], fvar[1], False))
        if adaptive:
            r.refine_adaptive(level)
        else:
            r.refine_uniform(level)
        ptex, u, v = shapes.uniform_locations(cage, 400, seed=48)
        rec = ref.limit_record(r, ptex, u, v, mode=mode, d1=d1, d2=d2)
        for k, a in rec.items():
            if isinstance(a, np.ndarray) and a.size == 0:
                continue
            out[f"{name}_{k}"] = np.asarray(a)
    out["cases"] = np.array([c[0] for c in cases])
    np.savez_compressed(path, **out)


REFERENCE = os.environ.get("OPENSUBDIV_SOURCE", "/root/reference")


def regression_shape(name):
    """A cage from the reference's regression shape `name` (regression/shapes/<name>.h: OBJ
    text in a C string -- v / f lines and crease, corner and interpolateboundary tags), read
    as data where the reference's sources are.  Boundary interpolation follows the
    regression tools (regression/common/far_utils.h:76-95): edge-only unless tagged."""
    path = os.path.join(REFERENCE, "regression", "shapes", name + ".h")
    src = open(path).read()
    body = src[src.index("std::string " + name):]
    # one string literal per line: "<obj line>\n"
    text = "".join(ln.strip()[1:-1] for ln in body.splitlines()[1:]
                   if ln.strip().startswith('"') and ln.strip().endswith('"'))
    text = text.replace("\\n", "\n")
    pos, vpf, fv, cv, cs, kv, ks = [], [], [], [], [], [], []
    boundary = 1  # Sdc VTX_BOUNDARY_EDGE_ONLY
    for line in text.split("\n"):
        t = line.split()
        if not t:
            continue
        if t[0] == "v":
            pos.append([float(x) for x in t[1:4]])
        elif t[0] == "f":
            idx = [int(x.split("/")[0]) - 1 for x in t[1:]]
            vpf.append(len(idx))
            fv.extend(idx)
        elif t[0] == "t":
            ni, nf = (int(x) for x in t[2].split("/")[:2])
            ints = [int(x) for x in t[3:3 + ni]]
            fls = [float(x) for x in t[3 + ni:3 + ni + nf]]
            if t[1] == "crease":
                for a, b in zip(ints[:-1], ints[1:]):
                    cv.append((a, b))
                    cs.append(fls[0])
            elif t[1] == "corner":
                kv.extend(ints)
                ks.extend([fls[0]] * len(ints))
            elif t[1] == "interpolateboundary":
                boundary = {0: 0, 1: 2, 2: 1}[ints[0]]
    scheme = shapes.LOOP if name.startswith("loop") else shapes.CATMARK
    cage = shapes.Cage(np.asarray(pos, np.float32), np.asarray(vpf, np.int32),
                       np.asarray(fv, np.int32), scheme=scheme, name=name)
    cage.crease_verts = np.asarray(cv, np.int32).reshape(-1, 2)
    cage.crease_sharpness = np.asarray(cs, np.float32)
    cage.corner_verts = np.asarray(kv, np.int32)
    cage.corner_sharpness = np.asarray(ks, np.float32)
    cage.boundary = boundary
    return cage


# The reference's regression shapes in the parity set: a valence-360 pole (stencils of 360+
# entries), boundaries with extraordinary vertices and both boundary interpolations, corner
# and crease tags, non-manifold edges, and Loop boundaries / poles.
REGRESSION_SHAPES = [
    ("catmark_pole360", 2, 3), ("catmark_xord_boundary", 3, 3), ("catmark_edgecorner", 3, 3),
    ("catmark_cube_corner2", 3, 3), ("catmark_cube_creases1", 3, 3),
    ("catmark_nonman_edges", 2, 3), ("loop_triangle_edgecorner", 3, 3),
    ("loop_xord_boundary", 3, 3), ("loop_pole64", 2, 3),
]


def regression_fixtures():
    for k, (name, ulevel, alevel) in enumerate(REGRESSION_SHAPES):
        cage = regression_shape(name)
        stencil_fixture(os.path.join(HERE, f"reg_{name}_uniform_L{ulevel}.npz"), cage, ulevel,
                        seed=100 + k, limit_level=alevel, nlimit=400)
        patch_fixture(os.path.join(HERE, f"reg_{name}_patches_L{alevel}.npz"), cage, alevel,
                      seed=200 + k, nq=1000)


def limit_pin_fixture(path):
    """Far::LimitStencilTableFactory on a uniform refiner (far/stencilTableFactory.cpp:411-662;
    the limit surface of a uniform table is bilinear over the last level's faces) at seeded
    locations: the table the workload generator's limit_stencil_table must reproduce."""
    cage = shapes.torus(16, 8, tri_fraction=0.1, crease_fraction=0.05, seed=3)
    level = 2
    r = ref.Refiner(cage).refine_uniform(level)
    face, u, v = shapes.uniform_locations(cage, 500, seed=4)
    lt = ref.limit_stencil_table(r, face, u, v, d1=True)
    out = dict(cage_arrays(cage))
    out.update(level=np.int32(level), face=face, u=u, v=v)
    for k in ("sizes", "offsets", "indices", "weights", "du_weights", "dv_weights"):
        out[k] = lt[k]
    np.savez_compressed(path, **out)


# ---- Bfr ----------------------------------------------------------------------------------

def bfr_tess_cases(seed=0):
    """(regular face size, face size, rates, facet size, preserve quads) for the pattern sweep:
    uniform rates, edge rates with and without inner rates, quads' two-inner-rate forms, the
    three facet options, N-gons to 13 sides, and invalid requests (a zero rate, a 2-gon, a
    quad of a triangle scheme)."""
    rng = np.random.default_rng(seed)
    opts = ((3, 0), (4, 0), (4, 1))
    cases = []
    for reg, sizes in ((4, (4, 3, 5, 6, 7, 8, 9, 10, 11, 13)), (3, (3,))):
        for N in sizes:
            for fs, pq in opts:
                for r in list(range(1, 11)) + [16, 31]:
                    cases.append((reg, N, [r], fs, pq))
                for _ in range(12):
                    kind = rng.integers(0, 4)
                    if kind == 0:
                        rates = rng.integers(1, 10, N)
                    elif kind == 1:
                        rates = rng.integers(1, 10, N + 1)
                    elif kind == 2 and N == 4:
                        rates = rng.integers(1, 10, rng.choice([2, 6]))
                    else:
                        base = int(rng.integers(2, 9))
                        rates = np.clip(base + rng.integers(-1, 2, N), 1, None)
                    cases.append((reg, N, [int(x) for x in rates], fs, pq))
    cases += [(4, 4, [0], 3, 0), (4, 2, [3], 3, 0), (3, 4, [3], 3, 0), (4, 5, [2, 0, 3, 1, 2], 4, 1)]
    return cases


def bfr_tess_fixture(path):
    """The reference's Bfr::Tessellation over the sweep of bfr_tess_cases: per case its
    validity, counts, coords (float32 bits) and facets."""
    cases = bfr_tess_cases()
    ro, rates, meta, co, coords, fo, facets = [0], [], [], [0], [], [0], []
    for reg, N, r, fs, pq in cases:
        rates += r
        ro.append(len(rates))
        t = ref.bfr_tess(reg, N, r, fs, pq)
        if t is None:
            meta.append((reg, N, fs, pq, 0, 0, 0, 0))
            co.append(co[-1])
            fo.append(fo[-1])
            continue
        cnt, c, f = t
        meta.append((reg, N, fs, pq, 1, int(cnt[2]), int(cnt[3]), 0))
        coords.append(c)
        facets.append(f.reshape(-1))
        co.append(co[-1] + len(c))
        fo.append(fo[-1] + f.size)
    np.savez_compressed(path, meta=np.asarray(meta, np.int32), rate_offsets=np.asarray(ro, np.int32),
                        rates=np.asarray(rates, np.int32), coord_offsets=np.asarray(co, np.int64),
                        coords=np.concatenate(coords).astype(np.float32),
                        facet_offsets=np.asarray(fo, np.int64),
                        facets=np.concatenate(facets).astype(np.int32))


def edge_rates(cage, rng, lo=1, hi=7):
    """Per-face edge rates from one seeded rate per mesh edge (shared edges get one rate, as
    rates derived from edge lengths do in the reference's tutorial 2.1)."""
    vpf = cage.verts_per_face
    fv = cage.face_verts
    start = np.concatenate([[0], np.cumsum(vpf)])
    rate_of = {}
    out = []
    for f in range(len(vpf)):
        vs = fv[start[f]:start[f + 1]]
        for i in range(len(vs)):
            e = (min(vs[i], vs[(i + 1) % len(vs)]), max(vs[i], vs[(i + 1) % len(vs)]))
            if e not in rate_of:
                rate_of[e] = int(rng.integers(lo, hi + 1))
            out.append(rate_of[e])
    return start.astype(np.int32), np.asarray(out, np.int32)


def bfr_mesh_fixture(path, cage, mode, facet_size=3, preserve_quads=False, seed=0, fvar=None):
    """Bfr tessellate-and-evaluate of every face (the reference's tutorial loop through
    Bfr::RefinerSurfaceFactory with its default approximation levels, Surface::Evaluate in
    float and double), plus the Far patch table the reference's Bfr regression pairs with those
    levels (isolation 6 / secondary 2, Gregory-basis end caps, infinitely sharp patches, no
    shared end-cap points, no legacy corner patches) and its PatchMap handles at every coord."""
    rng = np.random.default_rng(seed)
    reg = 3 if cage.scheme == shapes.LOOP else 4
    nf = len(cage.verts_per_face)
    if mode[0] == "u":
        ro = np.arange(nf + 1, dtype=np.int32)
        rates = np.full(nf, int(mode[1:]), np.int32)
    else:
        ro, rates = edge_rates(cage, rng)
    rf = None if fvar is None else (fvar[0], fvar[1], False)
    rec = ref.bfr_mesh_record(ref.Refiner(cage, fvar=rf), cage.positions, ro, rates, facet_size,
                              preserve_quads, uvs=None if fvar is None else fvar[2])
    r = ref.Refiner(cage, fvar=rf).refine_adaptive_levels(6, 2, True)
    p = ref.Patches(r, endcap=3, max_isolation=6, inf_sharp=True, share_endcap_points=False,
                    legacy_sharp_corners=False)
    nc = cage.num_vertices
    ns = len(p.st["sizes"])
    buf = np.zeros((nc + ns) * 3, np.float32)
    buf[: nc * 3] = cage.positions.reshape(-1)
    assert ref.cpu_eval_stencils(buf, (0, 3, 3), [buf], [(nc * 3, 3, 3)], p.st["sizes"],
                                 p.st["offsets"], p.st["indices"], [p.st["weights"]], 0, ns)
    sizes = cage.verts_per_face
    ptex = np.concatenate([[0], np.cumsum(np.where(sizes == reg, 1, sizes))]).astype(np.int64)
    co = rec["coord_offsets"]
    qf, qs, qt = [], [], []
    for f in range(nf):
        if co[f + 1] == co[f]:
            continue
        sub, st = ref.bfr_subface(reg, int(sizes[f]), rec["coords"][co[f]:co[f + 1]])
        qf.append(ptex[f] + sub)
        qs.append(st[:, 0])
        qt.append(st[:, 1])
    qf = np.concatenate(qf).astype(np.int32)
    qs = np.concatenate(qs).astype(np.float32)
    qt = np.concatenate(qt).astype(np.float32)
    handles, found = p.find_patches(qf, qs.astype(np.float64), qt.astype(np.float64))
    out = dict(cage_arrays(cage))
    out.update(regular_face_size=np.int32(reg), rate_offsets=ro, rates=rates,
               facet_size=np.int32(facet_size), preserve_quads=np.int32(preserve_quads),
               arrays=p.arrays, patch_indices=p.indices, params=p.params, src=buf,
               triangular=np.int32(reg == 3), ptex_offsets=ptex,
               coord_offsets=co, facet_offsets=rec["facet_offsets"], valid=rec["valid"],
               regular=rec["regular"], coords=rec["coords"], facets=rec["facets"],
               out6=rec["f32"], out6_fp64=rec["f64"], q_face=qf, q_s=qs, q_t=qt,
               q_handles=handles, q_found=found)
    if fvar is not None:
        # face-varying channel 0: the Far table's fvar patches and their points (the channel's
        # values, refined, then its local points), and Bfr's face-varying surfaces at the coords
        fa, fi, fp = p.fvar(0)
        fst = p.fvar_stencils(r, 0)
        nv = fvar[0]
        fbuf = np.zeros((nv + len(fst["sizes"])) * 2, np.float32)
        fbuf[: nv * 2] = np.asarray(fvar[2], np.float32).ravel()
        assert ref.cpu_eval_stencils(fbuf, (0, 2, 2), [fbuf], [(nv * 2, 2, 2)], fst["sizes"],
                                     fst["offsets"], fst["indices"], [fst["weights"]], 0,
                                     len(fst["sizes"]))
        out.update(fvar_arrays=fa, fvar_indices=fi, fvar_params=fp, fvar_src=fbuf,
                   uv_values=np.asarray(fvar[2], np.float32), uv3=rec["uv"])
    np.savez_compressed(path, **out)


BFR_MESHES = [
    ("catmark_nonquads", "u5", 3, 0), ("catmark_nonquads", "e", 4, 1),
    ("catmark_xord_boundary", "u4", 4, 1), ("catmark_edgecorner", "e", 3, 0),
    ("catmark_smoothtris0", "u3", 3, 0), ("catmark_gregory_test1", "e", 4, 0),
    ("loop_xord_boundary", "u5", 3, 0), ("loop_xord_boundary", "e", 4, 0),
]


def bfr_fixtures():
    bfr_tess_fixture(os.path.join(HERE, "bfr_tess_patterns.npz"))
    for k, (name, mode, fs, pq) in enumerate(BFR_MESHES):
        bfr_mesh_fixture(os.path.join(HERE, f"bfr_{name}_{mode}_f{fs}{'q' if pq else ''}.npz"),
                         regression_shape(name), mode, fs, pq, seed=300 + k)
    tor = shapes.torus(16, 8, tri_fraction=0.1, crease_fraction=0.05, seed=3)
    bfr_mesh_fixture(os.path.join(HERE, "bfr_torus16x8_e_f3.npz"), tor, "e", 3, 0, seed=320)
    ico = shapes.icosphere(1, noise=0.005, seed=3)
    bfr_mesh_fixture(os.path.join(HERE, "bfr_icosphere1_u6_f3.npz"), ico, "u6", 3, 0, seed=321)
    # face-varying UVs with seams (the reference's tutorial 1.3): Catmark with triangles, Loop
    ftor = shapes.torus(12, 8, tri_fraction=0.1, crease_fraction=0.05, seed=31, noise=0.01)
    bfr_mesh_fixture(os.path.join(HERE, "bfr_torus12x8_uv_e_f3.npz"), ftor, "e", 3, 0, seed=322,
                     fvar=uv_seams(ftor, 12, 8) + (uv_grid(12, 8),))
    fltor = shapes.torus(12, 8, seed=33, noise=0.01, scheme=shapes.LOOP)
    bfr_mesh_fixture(os.path.join(HERE, "bfr_looptorus12x8_uv_u4_f3.npz"), fltor, "u4", 3, 0,
                     seed=323, fvar=uv_seams(fltor, 12, 8) + (uv_grid(12, 8),))


def bfr_fixture_cage(key):
    """The cage a Bfr mesh fixture (bfr_<name>_<mode>_f<n>[q]) was written from, with the
    boundary and corner settings the fixture arrays do not carry."""
    for name, mode, fs, pq in BFR_MESHES:
        if key == f"bfr_{name}_{mode}_f{fs}{'q' if pq else ''}":
            return regression_shape(name)
    others = {
        "bfr_torus16x8_e_f3": lambda: shapes.torus(16, 8, tri_fraction=0.1,
                                                   crease_fraction=0.05, seed=3),
        "bfr_icosphere1_u6_f3": lambda: shapes.icosphere(1, noise=0.005, seed=3),
        "bfr_torus12x8_uv_e_f3": lambda: shapes.torus(12, 8, tri_fraction=0.1,
                                                      crease_fraction=0.05, seed=31, noise=0.01),
        "bfr_looptorus12x8_uv_u4_f3": lambda: shapes.torus(12, 8, seed=33, noise=0.01,
                                                           scheme=shapes.LOOP),
    }
    return others[key]()


def bfr_share_fixture(path):
    """The reference's tessellation with shared vertex and edge points (its tutorial 2.2
    bookkeeping over Bfr::Tessellation, through ref_bfr_share) on the cage and rates of every
    Bfr mesh fixture: per fixture the facets as point indices, the first point of each face
    and the coord each point is evaluated at."""
    out = {}
    for name in sorted(os.listdir(HERE)):
        if not (name.startswith("bfr_") and name.endswith(".npz")) or name in (
                "bfr_share.npz", "bfr_tess_patterns.npz", "bfr_stencils.npz"):
            continue
        d = np.load(os.path.join(HERE, name))
        cage = bfr_fixture_cage(name[:-4])
        assert np.array_equal(cage.face_verts, d["face_verts"])
        co, fo = d["coord_offsets"], d["facet_offsets"]
        facets, po, src = ref.bfr_share(ref.Refiner(cage), d["rate_offsets"], d["rates"],
                                        int(co[-1]), int(fo[-1]), int(d["facet_size"]),
                                        bool(d["preserve_quads"]))
        key = name[:-4]
        out[key + "__facets"] = facets
        out[key + "__point_offsets"] = po
        out[key + "__point_sources"] = src
    np.savez_compressed(path, **out)


BFR_STENCIL_MESHES = ["bfr_catmark_nonquads_u5_f3", "bfr_catmark_xord_boundary_u4_f4q",
                      "bfr_catmark_gregory_test1_e_f4", "bfr_loop_xord_boundary_u5_f3",
                      "bfr_torus16x8_e_f3"]


def bfr_stencil_fixture(path):
    """Bfr::Surface::EvaluateStencil (P, Du, Dv over mesh vertices) at every coord of the
    reference's tessellate loop, for some of the Bfr mesh fixtures, with the Far stencils of
    the paired patch table's points beyond the cage (refined and local points: the rows of the
    fixture's source buffer after the cage points)."""
    out = {}
    for key in BFR_STENCIL_MESHES:
        d = np.load(os.path.join(HERE, key + ".npz"))
        cage = bfr_fixture_cage(key)
        r = ref.Refiner(cage).refine_adaptive_levels(6, 2, True)
        p = ref.Patches(r, endcap=3, max_isolation=6, inf_sharp=True, share_endcap_points=False,
                        legacy_sharp_corners=False)
        assert np.array_equal(p.indices, d["patch_indices"])
        st = p.st
        bfr = ref.bfr_stencils(ref.Refiner(cage), d["rate_offsets"], d["rates"],
                               int(d["coord_offsets"][-1]), int(d["facet_size"]),
                               bool(d["preserve_quads"]))
        for k in ("sizes", "offsets", "indices", "weights"):
            out[f"{key}__st_{k}"] = np.asarray(st[k])
        for k in ("sizes", "indices", "wP", "wDu", "wDv"):
            out[f"{key}__bfr_{k}"] = bfr[k]
        # varying surfaces (InitVaryingSurface): seeded values per vertex, Far's varying
        # patches and varying stencils of the same refinement, and Bfr's values at every coord
        rng = np.random.default_rng(409 + 17 * BFR_STENCIL_MESHES.index(key))
        vals = rng.uniform(-1, 1, (cage.num_vertices, 3)).astype(np.float32)
        va, vi = p.varying()
        vst = ref.stencil_table_mode(r, mode=ref.INTERPOLATE_VARYING)
        out[f"{key}__var_values"] = vals
        out[f"{key}__var_arrays"] = va
        out[f"{key}__var_indices"] = vi
        for k in ("sizes", "offsets", "indices", "weights"):
            out[f"{key}__var_st_{k}"] = np.asarray(vst[k])
        # tutorial 2.1's limit option: rates from the limit positions at the face corners
        ext = float((cage.positions.max(0) - cage.positions.min(0)).max())
        lr, lp = ref.bfr_limit_rates(ref.Refiner(cage), cage.positions, len(cage.face_verts),
                                     ext / 40.0, 10)
        out[f"{key}__limit_rates"] = lr
        out[f"{key}__limit_points"] = lp
        out[f"{key}__var_bfr"] = ref.bfr_varying(
            ref.Refiner(cage), d["rate_offsets"], d["rates"], int(d["coord_offsets"][-1]), vals,
            int(d["facet_size"]), bool(d["preserve_quads"]))
    np.savez_compressed(path, **out)


LARGE = os.path.join(HERE, "large")


def large_patch_workload(path, cage, level):
    """A full-size EvalPatches workload from the reference's own Far: the adaptive patch table
    (isolation `level`, Gregory-basis end caps) flattened as Osd::CpuPatchTable, and the source
    buffer [cage points; refined points of every level; local points] computed with
    Osd::CpuEvaluator from Far's stencils.  Too large to commit: written under large/ (kept
    out of git) where the reference is available, for the benchmark and the full-size GPU
    parity test."""
    r = ref.Refiner(cage)
    r.refine_adaptive(level)
    p = ref.Patches(r, endcap=3, max_isolation=level)
    nc = cage.num_vertices
    ns = len(p.st["sizes"])
    buf = np.zeros((nc + ns) * 3, np.float32)
    buf[: nc * 3] = cage.positions.reshape(-1)
    ref.omp_set_threads(os.cpu_count() or 1)
    assert ref.cpu_eval_stencils(buf, (0, 3, 3), [buf], [(nc * 3, 3, 3)], p.st["sizes"],
                                 p.st["offsets"], p.st["indices"], [p.st["weights"]], 0, ns,
                                 omp=True)
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp.npz"
    np.savez_compressed(tmp, positions=cage.positions, level=np.int32(level), arrays=p.arrays,
             patch_indices=p.indices, params=p.params, src=buf,
             num_ptex=np.int32(r.num_ptex_faces()),
             triangular=np.int32(cage.scheme == shapes.LOOP))
    os.replace(tmp, path)


def large_bfr_workload(path, cage, rate=5, sample=0.02, seed=7):
    """The Bfr benchmark's Far table for the full-size torus: the approximation of
    Bfr::SurfaceFactory's defaults as the reference's Bfr regression builds it (adaptive
    isolation 6 for sharp and 2 for smooth features, Gregory-basis end caps, infinitely sharp
    patches, no shared end-cap points, no legacy corner patches) with its source points, plus
    the reference's Bfr tessellate-and-evaluate of a seeded `sample` of the faces at `rate`
    (the others rate 0, skipped) for the full-size parity test."""
    r = ref.Refiner(cage).refine_adaptive_levels(6, 2, True)
    p = ref.Patches(r, endcap=3, max_isolation=6, inf_sharp=True, share_endcap_points=False,
                    legacy_sharp_corners=False)
    nc = cage.num_vertices
    ns = len(p.st["sizes"])
    buf = np.zeros((nc + ns) * 3, np.float32)
    buf[: nc * 3] = cage.positions.reshape(-1)
    ref.omp_set_threads(os.cpu_count() or 1)
    assert ref.cpu_eval_stencils(buf, (0, 3, 3), [buf], [(nc * 3, 3, 3)], p.st["sizes"],
                                 p.st["offsets"], p.st["indices"], [p.st["weights"]], 0, ns,
                                 omp=True)
    nf = len(cage.verts_per_face)
    rng = np.random.default_rng(seed)
    rates = np.where(rng.random(nf) < sample, rate, 0).astype(np.int32)
    rec = ref.bfr_mesh_record(ref.Refiner(cage), cage.positions,
                              np.arange(nf + 1, dtype=np.int32), rates)
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp.npz"
    np.savez_compressed(tmp, positions=cage.positions, verts_per_face=cage.verts_per_face,
                        face_verts=cage.face_verts, arrays=p.arrays, patch_indices=p.indices, params=p.params, src=buf,
                        triangular=np.int32(0), rate=np.int32(rate), sample_rates=rates,
                        sample_coord_offsets=rec["coord_offsets"], sample_coords=rec["coords"],
                        sample_facets=rec["facets"], sample_out3=rec["f32"][:3])
    os.replace(tmp, path)


def large_bfr_stencil_workload(path, cage):
    """The Bfr limit-stencil benchmark's inputs: the Far table of Bfr::SurfaceFactory's default
    approximation for `cage` (as large_bfr_workload builds it), its source points, and Far's
    stencils of the refined and local points (the rows after the cage points) over the cage:
    the base GB300TessellationStencils composes over.  Written under large/ (kept out of git)."""
    r = ref.Refiner(cage).refine_adaptive_levels(6, 2, True)
    p = ref.Patches(r, endcap=3, max_isolation=6, inf_sharp=True, share_endcap_points=False,
                    legacy_sharp_corners=False)
    nc = cage.num_vertices
    ns = len(p.st["sizes"])
    buf = np.zeros((nc + ns) * 3, np.float32)
    buf[: nc * 3] = cage.positions.reshape(-1)
    ref.omp_set_threads(os.cpu_count() or 1)
    assert ref.cpu_eval_stencils(buf, (0, 3, 3), [buf], [(nc * 3, 3, 3)], p.st["sizes"],
                                 p.st["offsets"], p.st["indices"], [p.st["weights"]], 0, ns,
                                 omp=True)
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp.npz"
    np.savez_compressed(tmp, positions=cage.positions, verts_per_face=cage.verts_per_face,
                        face_verts=cage.face_verts, arrays=p.arrays, patch_indices=p.indices,
                        params=p.params, src=buf, st_sizes=p.st["sizes"],
                        st_offsets=p.st["offsets"], st_indices=p.st["indices"],
                        st_weights=p.st["weights"])
    os.replace(tmp, path)


def large_workloads():
    """The EvalPatches benchmark tables: the plain-method torus (512 x 256, R = 1, r = 0.3,
    seeded 5% triangles and 2% creases U[0, 4]; the cage of the stencil benchmark) and the
    Loop icosphere subdivided 6 times (40,962 points, N(0, 0.005) noise), both at adaptive
    isolation level 4 with Gregory-basis end caps."""
    torus = shapes.torus(512, 256, R=1.0, r=0.3, tri_fraction=0.05, crease_fraction=0.02,
                         max_sharpness=4.0, seed=2024)
    large_patch_workload(os.path.join(LARGE, "torus512x256_adaptiveL4.npz"), torus, 4)
    ico = shapes.icosphere(6, noise=0.005, seed=3)
    large_patch_workload(os.path.join(LARGE, "icosphere6_loop_adaptiveL4.npz"), ico, 4)
    large_bfr_workload(os.path.join(LARGE, "torus512x256_bfr.npz"), torus)
    large_bfr_stencil_workload(os.path.join(LARGE, "torus256x128_bfr_stencils.npz"),
                               shapes.torus(256, 128, R=1.0, r=0.3, tri_fraction=0.05,
                                            crease_fraction=0.02, max_sharpness=4.0, seed=2024))


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "large":
        if not ref.available():
            raise SystemExit("oracle/_ref/libosdref.so missing: run `make -C oracle ref` first")
        large_workloads()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "regression":
        regression_fixtures()
        limit_pin_fixture(os.path.join(HERE, "uniform_limit_pin.npz"))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "bfr":
        bfr_fixtures()
        bfr_share_fixture(os.path.join(HERE, "bfr_share.npz"))
        bfr_stencil_fixture(os.path.join(HERE, "bfr_stencils.npz"))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "bfr-share":
        bfr_share_fixture(os.path.join(HERE, "bfr_share.npz"))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "bfr-stencils":
        bfr_stencil_fixture(os.path.join(HERE, "bfr_stencils.npz"))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "bfr-stencils-large":
        large_bfr_stencil_workload(
            os.path.join(LARGE, "torus256x128_bfr_stencils.npz"),
            shapes.torus(256, 128, R=1.0, r=0.3, tri_fraction=0.05, crease_fraction=0.02,
                         max_sharpness=4.0, seed=2024))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "bfr-large":
        torus = shapes.torus(512, 256, R=1.0, r=0.3, tri_fraction=0.05, crease_fraction=0.02,
                             max_sharpness=4.0, seed=2024)
        large_bfr_workload(os.path.join(LARGE, "torus512x256_bfr.npz"), torus)
        return
    if len(sys.argv) > 1 and sys.argv[1] == "factory":
        factory_fixture(os.path.join(HERE, "factory_masks.npz"))
        factory_limit_fixture(os.path.join(HERE, "factory_limit.npz"))
        return
    if not ref.available():
        raise SystemExit("oracle/_ref/libosdref.so missing: run `make -C oracle ref` first")
    g = HERE
    # Config-1 family: noisy 8x8-per-face cube, Catmull-Clark.
    cube = shapes.cube(8, noise=0.01, seed=1)
    stencil_fixture(os.path.join(g, "cube8_uniform_L3.npz"), cube, 3, seed=11,
                    limit_level=3, nlimit=600)
    # Config-2 family at reduced size: torus with triangles and semi-sharp creases.
    tor = shapes.torus(32, 16, tri_fraction=0.05, crease_fraction=0.02, seed=2)
    stencil_fixture(os.path.join(g, "torus32x16_uniform_L2.npz"), tor, 2, seed=12,
                    limit_level=4, nlimit=600)
    # Loop uniform stencils (icosphere and creased all-triangle torus).
    ico = shapes.icosphere(2, noise=0.005, seed=3)
    stencil_fixture(os.path.join(g, "icosphere2_uniform_L2.npz"), ico, 2, seed=13)
    ltor = shapes.torus(12, 8, crease_fraction=0.05, seed=4, scheme=shapes.LOOP)
    stencil_fixture(os.path.join(g, "looptorus12x8_uniform_L2.npz"), ltor, 2, seed=14)
    # Config-3 family: adaptive patch tables with Gregory-basis end caps.
    patch_fixture(os.path.join(g, "torus32x16_patches_L4.npz"), tor, 4, seed=21)
    patch_fixture(os.path.join(g, "icosphere2_patches_L3.npz"), ico, 3, seed=22)
    # Varying and face-varying tables: tori with UV seams (non-linear face-varying patches)
    ftor = shapes.torus(12, 8, tri_fraction=0.1, crease_fraction=0.05, seed=31, noise=0.01)
    patch_fixture(os.path.join(g, "torus12x8_fvar_patches_L3.npz"), ftor, 3, seed=32,
                  nq=1500, fvar=uv_seams(ftor, 12, 8) + (uv_grid(12, 8),))
    fltor = shapes.torus(12, 8, seed=33, noise=0.01, scheme=shapes.LOOP)
    patch_fixture(os.path.join(g, "looptorus12x8_fvar_patches_L3.npz"), fltor, 3, seed=34,
                  nq=1500, fvar=uv_seams(fltor, 12, 8) + (uv_grid(12, 8),))
    # Boundaries: open grids (B-spline and box-spline boundary masks).
    patch_fixture(os.path.join(g, "grid6_patches_L3.npz"), shapes.grid(6, 6, seed=5), 3,
                  seed=23, nq=1500)
    patch_fixture(os.path.join(g, "trigrid6_patches_L3.npz"),
                  shapes.grid(6, 6, seed=6, scheme=shapes.LOOP), 3, seed=24, nq=1500)
    # B-spline end caps and uniform (linear) tables.
    patch_fixture(os.path.join(g, "cube8_patches_bspline_L2.npz"), cube, 2, seed=25, nq=1500,
                  endcap=2)
    patch_fixture(os.path.join(g, "cube8_uniform_quads_L1.npz"), cube, 1, seed=26, nq=1500,
                  adaptive=False)
    patch_fixture(os.path.join(g, "icosphere2_uniform_tris_L1.npz"), ico, 1, seed=27,
                  nq=1500, adaptive=False)
    factory_fixture(os.path.join(g, "factory_masks.npz"))
    factory_limit_fixture(os.path.join(g, "factory_limit.npz"))
    # the reference's regression shapes, and the uniform-refiner limit-stencil pin
    regression_fixtures()
    limit_pin_fixture(os.path.join(g, "uniform_limit_pin.npz"))
    for f in sorted(os.listdir(g)):
        if f.endswith(".npz"):
            print(f"{f:40s} {os.path.getsize(os.path.join(g, f)) / 1024:8.1f} KiB")


if __name__ == "__main__":
    main()
