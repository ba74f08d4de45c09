"""Seeded synthetic workloads with the shapes of the evaluation benchmarks.

``refine_and_limit_torus`` is the plain-method workload: a 512 x 256 quad torus (R = 1,
r = 0.3, 131,072 control vertices) with a seeded 5% of its quads split into two triangles
along a random diagonal and a seeded 2% of its edges given sharpness U[0, 4]; Catmull-Clark
uniform refinement to level 3 (factorized stencils of the level-3 vertices only), evaluated
on 8 interleaved float32 primvars (xyz + 5 channels U[-1, 1]); plus limit stencils with
du/dv weights at 1M seeded (ptex face, u, v) locations on the same refiner.

``refine_cube`` is the CPU-runnable case: the unit cube with 8 x 8 quads per face (386
control vertices), N(0, 0.01) noise, Catmull-Clark level 4, xyz.
"""
from __future__ import annotations

import numpy as np

from . import shapes
from .topology import UniformRefiner


def stencil_bytes(n_stencils, nnz, length, n_cv, n_weight_arrays=1, n_outputs=1):
    """Algorithmic bytes of one EvalStencils pass: sizes + offsets (8 B per stencil), indices
    and weight arrays (4 B each per entry), outputs (4 B x length per stencil per output) and
    the source rows read once (4 B x length per control vertex)."""
    return (8 * n_stencils + 4 * nnz * (1 + n_weight_arrays) + 4 * length * n_stencils * n_outputs
            + 4 * length * n_cv)


def refine_and_limit_torus(nu=512, nv=256, level=3, n_limit=1_000_000, length=8, seed=2024):
    cage = shapes.torus(nu, nv, R=1.0, r=0.3, tri_fraction=0.05, crease_fraction=0.02,
                        max_sharpness=4.0, seed=seed)
    rng = np.random.default_rng(seed + 1)
    ncv = cage.num_vertices
    src = np.concatenate([cage.positions,
                          rng.uniform(-1, 1, (ncv, length - 3)).astype(np.float32)], 1)
    refiner = UniformRefiner(cage, level)
    refine = refiner.stencil_table()
    face, u, v = shapes.uniform_locations(cage, n_limit, seed=seed + 2)
    limit = refiner.limit_stencil_table(face, u, v)
    return dict(name=f"torus{nu}x{nv}_catmark_L{level}_{length}pv_limit{n_limit // 1000}k",
                cage=cage, src=np.ascontiguousarray(src.ravel()), length=length, refine=refine,
                limit=limit, level=level)


def instanced_patch_table(table, copies):
    """`copies` disjoint instances of a flattened Far patch table (Osd::CpuPatchTable layout;
    `table` maps arrays, patch_indices, params, src, num_ptex, triangular to arrays): arrays
    stay grouped by patch type, every copy's control indices are offset by the source size and
    its ptex faces by the ptex count.  Returns arrays, indices, params, the source points (copy
    c displaced by 3c along x), the ptex face count and whether the table is triangular."""
    z = table
    arr, idx, par, src = z["arrays"], z["patch_indices"], z["params"], z["src"].reshape(-1, 3)
    nsrc, nptex = len(src), int(z["num_ptex"])
    arrays, indices, params = [], [], []
    ibase = pbase = 0
    for a in arr:
        t_reg, t_irr, npatch, ib, stride, pb = (int(x) for x in a)
        block = idx[ib: ib + npatch * stride]
        pblock = par[pb: pb + npatch]
        arrays.append([t_reg, t_irr, npatch * copies, ibase, stride, pbase])
        for c in range(copies):
            indices.append(block + c * nsrc)
            p = pblock.copy()
            face = (p[:, 0] & 0xFFFFFFF) + c * nptex
            p[:, 0] = (p[:, 0] & ~0xFFFFFFF) | face
            params.append(p)
        ibase += npatch * stride * copies
        pbase += npatch * copies
    shift = np.zeros((copies, 1, 3), np.float32)
    shift[:, 0, 0] = np.arange(copies, dtype=np.float32) * 3.0
    srcs = (src[None, :, :] + shift).reshape(-1)
    return (np.asarray(arrays, np.int32), np.concatenate(indices).astype(np.int32),
            np.concatenate(params).astype(np.int32), np.ascontiguousarray(srcs, np.float32),
            nptex * copies, bool(z["triangular"]))


def eval_patches_points(table, name, n_points=4_000_000, seed=7):
    """EvalPatches workload over a flattened Far patch table (a mapping with arrays,
    patch_indices, params, src, num_ptex, triangular): n_points uniform (ptex face, u, v)
    locations, folded into the triangle (u + v <= 1) for triangular tables."""
    tri = bool(table["triangular"])
    nptex = int(table["num_ptex"])
    rng = np.random.default_rng(seed)
    face = rng.integers(0, nptex, n_points).astype(np.int32)
    u = rng.random(n_points).astype(np.float32)
    v = rng.random(n_points).astype(np.float32)
    if tri:
        fold = u + v > 1.0
        u[fold], v[fold] = 1.0 - u[fold], 1.0 - v[fold]
    return dict(name=f"{name}_{n_points / 1e6:g}Mpts", arrays=np.asarray(table["arrays"]),
                indices=np.asarray(table["patch_indices"]), params=np.asarray(table["params"]),
                src=np.ascontiguousarray(table["src"], np.float32), length=3, num_ptex=nptex,
                triangular=tri, face=face, u=u, v=v)


def instanced_points(table, name, target_patches, n_points=4_000_000, seed=7,
                     count_type=None):
    """eval_patches_points over `table` instanced to `target_patches` patches (of type
    `count_type` only, when given): a stand-in of a large table's size built from a small one."""
    arr = np.asarray(table["arrays"])
    per = int(arr[:, 2].sum() if count_type is None else arr[arr[:, 0] == count_type, 2].sum())
    copies = max(1, round(target_patches / per))
    arrays, indices, params, src, nptex, tri = instanced_patch_table(table, copies)
    w = eval_patches_points(dict(arrays=arrays, patch_indices=indices, params=params, src=src,
                                 num_ptex=nptex, triangular=tri), f"{name}_x{copies}",
                            n_points, seed)
    w["copies"] = copies
    return w


# FP32 operations of one EvalPatches point with all six outputs, per basis (an FMA counts 2),
# counted from the kernels' arithmetic in csrc/patch_basis.cuh: (weights, per primvar element).
#   REGULAR: two cubic B-spline curves (value, d, dd) ~66 + normalisation 4; per element 16
#     local-origin subtractions, 4 rows x (3 x 4 FMA row sums + 6 FMA accumulations), the
#     origin added back, 6 derivative scales: 16 + 144 + 1 + 6.
#   GREGORY_BASIS: two cubic Bezier curves ~50, 4 rational blend weights ~16; per element 20
#     subtractions, 4 blended pairs x 4, the same 4 x 36 row sums, origin, scales: 20+16+144+7.
#   LOOP: 12 monomials, 351 non-zero box-spline coefficients x 2, 48 constant scales; per
#     element 12 subtractions, 6 x 12 FMA, origin, scales: 12 + 144 + 7.
#   GREGORY_TRIANGLE: 3 blend pairs ~20, 6 quartic Bezier-triangle weight sets ~270; per element
#     18 subtractions, 3 blends x 3, 6 x 15 FMA, origin, scales: 18 + 9 + 180 + 7.
#   QUADS / TRIANGLES: bilinear / linear weights and 4 / 3 rows.
PATCH_FLOPS = {6: (70, 167), 9: (66, 187), 5: (762, 163), 10: (290, 214), 3: (10, 27),
               4: (4, 14)}
PATCH_CVS = {6: 16, 9: 20, 5: 12, 10: 18, 3: 4, 4: 3}


def point_types(coords, arrays, params):
    """Basis type of every evaluated point (-1 for PatchMap misses): the array's regular
    descriptor when the patch's param marks it regular, its irregular descriptor otherwise."""
    c = np.asarray(coords).reshape(-1, 5)
    arrays = np.asarray(arrays).reshape(-1, 6)
    params = np.asarray(params).reshape(-1, 3)
    hit = c[:, 0] >= 0
    t = np.full(len(c), -1, np.int64)
    ai, pi = c[hit, 0], c[hit, 1]
    regular = (params[pi, 1] >> 5) & 1
    t[hit] = np.where(regular == 1, arrays[ai, 0], arrays[ai, 1])
    return t


def patch_flops(types, length):
    """FP32 operations of one EvalPatches pass with all six outputs (PATCH_FLOPS)."""
    total = 0
    for ty, (w, e) in PATCH_FLOPS.items():
        total += int((types == ty).sum()) * (w + e * length)
    return total


def patch_gathered_bytes(types, length, n_outputs):
    """As-gathered bytes of one EvalPatches pass: every point's coord (20 B), array record
    (24 B), param (12 B), index row (4 B per control point), every control point row it
    reads (4 B x length each, re-reads counted) and its outputs."""
    total = 0
    for ty, ncv in PATCH_CVS.items():
        k = int((types == ty).sum())
        total += k * (20 + 24 + 12 + 4 * ncv + 4 * length * ncv + 4 * length * n_outputs)
    return total


def patch_bytes(n_points, length, n_outputs, n_src, touched_patches, cvs_per_patch):
    """Unique-bytes model of one EvalPatches pass: coords (20 B per point), outputs
    (4 B x length x outputs per point), touched patches' index rows and params
    (4 B x CVs + 12 B) and the source once (4 B x length per point)."""
    return (20 * n_points + 4 * length * n_outputs * n_points
            + touched_patches * (4 * cvs_per_patch + 12) + 4 * length * n_src)


def refine_cube(n=8, level=4, seed=1):
    cage = shapes.cube(n, noise=0.01, seed=seed)
    refine = UniformRefiner(cage, level).stencil_table()
    return dict(name=f"cube{n}_catmark_L{level}_xyz", cage=cage,
                src=np.ascontiguousarray(cage.positions.ravel()), length=3, refine=refine,
                level=level)


def _population_specs(n_meshes, cv_min, cv_max, seed):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_meshes):
        loop = bool(rng.random() < 0.3)
        kind = "torus" if rng.random() < 0.5 else "cube"
        cv = float(np.exp(rng.uniform(np.log(cv_min), np.log(cv_max))))
        specs.append(dict(index=i, loop=loop, kind=kind, cv=cv, level=int(rng.integers(1, 5)),
                          length=int(rng.integers(3, 13)),
                          phase=float(rng.uniform(0.0, 2.0 * np.pi))))
    return specs


def _population_mesh(sp, seed):
    """The cage and source values of one population mesh (without its table)."""
    scheme = shapes.LOOP if sp["loop"] else shapes.CATMARK
    s = seed * 1000 + sp["index"]
    if sp["kind"] == "torus":
        nv = max(3, int(round(np.sqrt(sp["cv"] / 2.0))))
        nu = max(3, int(round(sp["cv"] / nv)))
        cage = shapes.torus(nu, nv, noise=0.005, seed=s, scheme=scheme)
    else:
        n = max(1, int(round(np.sqrt(max(sp["cv"] - 2.0, 6.0) / 6.0))))
        cage = shapes.cube(n, noise=0.01, seed=s, scheme=scheme)
    r = np.random.default_rng(s + 1)
    ncv = cage.num_vertices
    src = np.concatenate([cage.positions,
                          r.uniform(-1, 1, (ncv, sp["length"] - 3)).astype(np.float32)], 1)
    return cage, dict(name=f"{cage.name}_{'loop' if sp['loop'] else 'catmark'}_L{sp['level']}",
                      scheme=scheme, level=sp["level"], length=sp["length"],
                      phase=sp["phase"], n_cv=ncv, src=np.ascontiguousarray(src.ravel()))


def batch_population(n_meshes=256, cv_min=500, cv_max=200_000, seed=4096, threads=None):
    """Meshes of uneven size for batched evaluation: procedural noisy tori or cubes (50/50)
    with control-vertex counts log-uniform in [cv_min, cv_max], 70% Catmull-Clark and 30%
    Loop (every quad split along a random diagonal), uniform refinement level uniform in
    {1, 2, 3, 4} (stencils of the finest level only) and 3-12 float32 primvars (xyz + U[-1, 1]
    channels), each with a seeded deformation phase.  Tables are generated on `threads` host
    threads (default: all cores), one mesh per thread.

    Returns a list of dicts: name, scheme, level, length, phase, n_cv, src (float32 n_cv x
    length, flattened), table (Far-layout arrays)."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    from .topology import load as _topo_load

    def build(sp):
        _topo_load().GB300TopologySetNumThreads(1)
        cage, m = _population_mesh(sp, seed)
        m["table"] = UniformRefiner(cage, sp["level"]).stencil_table()
        return m

    _topo_load()  # load once before the workers start
    with ThreadPoolExecutor(threads or os.cpu_count()) as ex:
        return list(ex.map(build, _population_specs(n_meshes, cv_min, cv_max, seed)))


def batch_population_masks(n_meshes=256, cv_min=500, cv_max=200_000, seed=4096, threads=None):
    """The same population as batch_population, each mesh with the Far-form subdivision masks
    of its levels instead of a table: masks = (number of control vertices, per-level masks),
    the input of the GPU stencil-table factory.  Host topology and masks are produced on
    `threads` host threads, largest meshes first, at most 2 x threads meshes ahead of the
    consumer (bounded host memory); meshes are yielded as they complete, each with its
    population `index`."""
    import os
    from concurrent.futures import FIRST_COMPLETED, ThreadPoolExecutor, wait

    from .topology import load as _topo_load

    def build(sp):
        _topo_load().GB300TopologySetNumThreads(1)
        cage, m = _population_mesh(sp, seed)
        m["index"] = sp["index"]
        m["masks"] = UniformRefiner(cage, sp["level"], stencils=False).factory_masks()
        return m

    _topo_load()
    threads = threads or os.cpu_count() or 1
    specs = sorted(_population_specs(n_meshes, cv_min, cv_max, seed),
                   key=lambda sp: -sp["cv"] * 4.0 ** sp["level"])
    with ThreadPoolExecutor(threads) as ex:
        it = iter(specs)
        pending = set()
        for sp in it:
            pending.add(ex.submit(build, sp))
            if len(pending) >= 2 * threads:
                break
        while pending:
            done, pending = wait(pending, return_when=FIRST_COMPLETED)
            for f in done:
                nxt = next(it, None)
                if nxt is not None:
                    pending.add(ex.submit(build, nxt))
                yield f.result()


def deform(base, phase, frame, amplitude=0.01):
    """Per-frame sinusoidal displacement of every control value: base + a sin(0.1 frame +
    phase + 7 base), with the mesh's phase (works on numpy arrays and torch tensors)."""
    lib = np if isinstance(base, np.ndarray) else __import__("torch")
    return base + amplitude * lib.sin(0.1 * frame + phase + 7.0 * base)


# ---- serving pool ----------------------------------------------------------------------------

def sort_entries(table):
    """Far-layout table with every stencil's entries in ascending control-index order (the
    device layout GB300StencilTableCreate uses; same stencils, better gather locality)."""
    sizes, offsets = table["sizes"], table["offsets"]
    row = np.repeat(np.arange(len(sizes)), sizes)
    pos = np.concatenate([np.arange(o, o + s) for o, s in zip(offsets, sizes)]) if len(sizes) \
        else np.zeros(0, np.int64)
    order = np.lexsort((table["indices"][pos], row))
    pos = pos[order]
    new_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int32)
    return dict(sizes=sizes.astype(np.int32), offsets=new_off,
                indices=table["indices"][pos].astype(np.int32),
                weights=table["weights"][pos].astype(np.float32))


def instance_table(table, copies, src_per_copy):
    """`copies` disjoint copies of a stencil table: copy c reads source rows offset by
    c * src_per_copy and produces rows c * numStencils + i."""
    n, nnz = len(table["sizes"]), len(table["indices"])
    c = np.arange(copies, dtype=np.int64)
    return dict(sizes=np.tile(table["sizes"], copies),
                offsets=(table["offsets"][None, :] + (c * nnz)[:, None]).astype(np.int32).ravel(),
                indices=(table["indices"][None, :] + (c * src_per_copy)[:, None])
                .astype(np.int32).ravel(),
                weights=np.tile(table["weights"], copies))


class ServingBase:
    """One base shape of the serving pool: an adaptive patch table of a small cage (a mapping
    with the cage -- positions, verts_per_face, face_verts, scheme, crease_verts,
    crease_sharpness -- the flattened Far patch table and its patch points' stencils over the
    cage: ps_sizes, ps_offsets, ps_indices, ps_weights), and uniform refinement tables of the
    same cage from the native generator (one per level, cached)."""

    def __init__(self, z):
        self.scheme = int(z["scheme"])
        self.table = {k: np.asarray(z[k]) for k in ("arrays", "patch_indices", "params", "src",
                                                     "num_ptex", "triangular")}
        self.cage = shapes.Cage(z["positions"], z["verts_per_face"], z["face_verts"],
                                scheme=int(z["scheme"]), name=f"base{int(z['scheme'])}")
        self.cage.crease_verts = z["crease_verts"]
        self.cage.crease_sharpness = z["crease_sharpness"]
        self.nc = len(z["positions"])
        self.ns = len(z["ps_sizes"])
        self.nptex = int(z["num_ptex"])
        self.triangular = bool(z["triangular"])
        # patch source of one copy = [cage points (identity stencils); patch points]
        eye = dict(sizes=np.ones(self.nc, np.int32), offsets=np.arange(self.nc, dtype=np.int32),
                   indices=np.arange(self.nc, dtype=np.int32), weights=np.ones(self.nc, np.float32))
        ps = dict(sizes=z["ps_sizes"], offsets=z["ps_offsets"] + self.nc, indices=z["ps_indices"],
                  weights=z["ps_weights"])
        self.pp = sort_entries({k: np.concatenate([eye[k], ps[k]]) for k in eye})
        self._refine = {}
        self._patch = {}

    def refine(self, level):
        if level not in self._refine:
            self._refine[level] = sort_entries(UniformRefiner(self.cage, level).stencil_table())
        return self._refine[level]

    def patch_table(self, copies):
        if copies not in self._patch:
            arrays, indices, params, _, nptex, tri = instanced_patch_table(self.table, copies)
            self._patch[copies] = (arrays, indices, params, nptex)
        return self._patch[copies]


def serving_pool(bases, n_topologies=1000, cv_min=500, cv_max=25_000, seed=5150):
    """Topologies for the serving loop, drawn like the batching population: CV counts
    log-uniform in [cv_min, cv_max], 70% Catmull-Clark / 30% Loop, uniform refinement level
    uniform in {1..4}, 3-12 float32 primvars.  Topology = `copies` instances of a base cage
    (`bases`: {shapes.CATMARK: ServingBase, shapes.LOOP: ServingBase}) with copies = CV
    target / base CVs rounded to a log-spaced set (so host tables are shared between
    topologies of the same (base, copies, level); every topology still has its own device copy
    when resident).  Each has a refine table at its level and limit tables (patch points as
    stencils over the cage's xyz + the instanced adaptive patch table)."""
    rng = np.random.default_rng(seed)
    steps = np.array([1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128, 192], np.int64)
    cache = {}
    pool = []
    for t in range(n_topologies):
        scheme = shapes.LOOP if rng.random() < 0.3 else shapes.CATMARK
        b = bases[scheme]
        cv = float(np.exp(rng.uniform(np.log(cv_min), np.log(cv_max))))
        copies = int(steps[np.argmin(np.abs(np.log(steps) - np.log(max(cv / b.nc, 1.0))))])
        level = int(rng.integers(1, 5))
        length = int(rng.integers(3, 13))
        key = (scheme, copies, level)
        if key not in cache:
            refine = instance_table(b.refine(level), copies, b.nc)
            arrays, pidx, params, nptex = b.patch_table(copies)
            pp = instance_table(b.pp, copies, b.nc)
            cache[key] = dict(refine=refine, limit=dict(
                pp_sizes=pp["sizes"], pp_offsets=pp["offsets"], pp_indices=pp["indices"],
                pp_weights=pp["weights"], arrays=arrays, patch_indices=pidx, params=params,
                triangular=b.triangular), num_ptex=nptex)
        c = cache[key]
        pool.append(dict(id=t, scheme=scheme, copies=copies, level=level, length=length,
                         num_control=copies * b.nc, refine=c["refine"], limit=c["limit"],
                         num_ptex=c["num_ptex"], base=b))
    return pool


def serving_control_values(topo, seed):
    """Deformed control values of a pool topology: the base cage positions of every copy
    (copy c shifted by 3c along x) plus U[-1, 1] channels, float32 [numControl x length]."""
    b = topo["base"]
    rng = np.random.default_rng(seed)
    pos = np.tile(b.cage.positions, (topo["copies"], 1)).astype(np.float64)
    pos[:, 0] += np.repeat(np.arange(topo["copies"]) * 3.0, b.nc)
    pos += rng.normal(0.0, 0.002, pos.shape)
    extra = rng.uniform(-1, 1, (len(pos), topo["length"] - 3))
    return np.ascontiguousarray(np.concatenate([pos, extra], 1).astype(np.float32).ravel())


def serving_queries(topo, n, seed):
    """n uniform (ptex face, u, v) queries (Loop: folded into u + v <= 1)."""
    rng = np.random.default_rng(seed)
    face = rng.integers(0, topo["num_ptex"], n).astype(np.int32)
    u = rng.random(n).astype(np.float32)
    v = rng.random(n).astype(np.float32)
    if topo["base"].triangular:
        f = u + v > 1.0
        u[f], v[f] = 1.0 - u[f], 1.0 - v[f]
    return face, u, v


# ---- Bfr tessellation ----------------------------------------------------------------------

def bfr_edge_length_rates(positions, verts_per_face, face_verts, interval, max_rate=64):
    """Per-face edge rates from control-hull edge lengths, the non-uniform scheme of the
    reference's Bfr tutorial 2.1 with its hull option (tutorials/bfr/tutorial_2_1/
    bfr_tutorial_2_1.cpp:121-166): an edge's length in float from the absolute coordinate
    differences of its two control points, its rate 1 + (int)(length / interval) capped at
    max_rate; both faces of an edge see the same length, so shared edges get one rate.
    Returns (rate_offsets, rates) with N rates per N-sided face (rates[i] for the edge from
    vertex i to i + 1)."""
    vpf = np.asarray(verts_per_face, np.int64)
    fv = np.asarray(face_verts, np.int64)
    start = np.concatenate([[0], np.cumsum(vpf)])
    nxt = np.arange(len(fv)) + 1
    last = start[1:] - 1
    nxt[last] = start[:-1]
    p = np.asarray(positions, np.float32)
    dv = np.abs(p[fv] - p[fv[nxt]])
    length = np.sqrt(dv[:, 0] * dv[:, 0] + dv[:, 1] * dv[:, 1] + dv[:, 2] * dv[:, 2])
    rates = np.minimum(1 + (length / np.float32(interval)).astype(np.int32), max_rate)
    return start.astype(np.int32), rates.astype(np.int32)


def bfr_tess_bytes(n_faces, n_coords, n_facets, facet_size, locate=True, uniform=True):
    """Algorithmic bytes of the tessellation kernels for a mesh: per face its size and (with
    per-face rates) its rate run, three offsets read twice; per coord the (u,v) pair written
    and, when located, a 20-byte PatchCoord; per facet its indices."""
    per_face = 4 + 3 * 8 * 2 + (0 if uniform else 4 * 5)
    return (per_face * n_faces + 8 * n_coords + (20 * n_coords if locate else 0)
            + 4 * facet_size * n_facets)


def face_edges(verts_per_face, face_verts):
    """Edge index of every face corner (the edge from corner i to corner i + 1), undirected
    edges numbered in order of first appearance, and the number of edges: the base level's
    face edges (Far::TopologyLevel::GetFaceEdges) for a mesh given as face vertices.  Shared
    tessellation points depend only on which corners name the same edge, not on its number."""
    vpf = np.asarray(verts_per_face, np.int64)
    fv = np.asarray(face_verts, np.int64)
    start = np.concatenate([[0], np.cumsum(vpf)])
    nxt = np.arange(len(fv)) + 1
    has = vpf > 0
    nxt[start[1:][has] - 1] = start[:-1][has]
    b = fv[nxt] if len(fv) else fv
    key = np.minimum(fv, b) * (int(fv.max(initial=0)) + 1) + np.maximum(fv, b)
    _, first, inv = np.unique(key, return_index=True, return_inverse=True)
    rank = np.empty(len(first), np.int64)
    rank[np.argsort(first)] = np.arange(len(first))
    return rank[inv].astype(np.int32), len(first)


def bfr_share_bytes(n_faces, n_corners, n_vertices, n_edges, n_facets, n_points, facet_size):
    """Algorithmic bytes of the shared-point pass: per face its size and three offsets; per
    corner its vertex and edge, read once; per vertex a 64-bit claim and its point, per edge a
    64-bit claim, its inside count and first point; per facet its indices read and rewritten;
    per point the source PatchCoord read and the point's PatchCoord written."""
    return (4 * n_faces + 3 * 8 * (n_faces + 1) + 8 * n_corners + 12 * n_vertices
            + 16 * n_edges + 2 * 4 * facet_size * n_facets + 40 * n_points)
