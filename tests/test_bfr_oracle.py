"""Pin the Bfr restatement (oracle/bfr_oracle.c) to the reference's Bfr.

tests/golden/bfr_tess_patterns.npz holds the reference's Bfr::Tessellation over a sweep of
faces, rates and options; tests/golden/bfr_<mesh>_*.npz the reference's Bfr tessellate-and-
evaluate loop over whole meshes (Bfr::RefinerSurfaceFactory + Tessellation + Surface::Evaluate)
with the Far patch table its Bfr regression pairs with the same approximation, and Far::PatchMap
handles at every coord (tests/golden/make_golden.py bfr).

The oracle must reproduce every coord bit for bit, every facet, the sub-face conversion bit for
bit and the PatchMap handles exactly; evaluating the Far table at the located coords must agree
with Bfr::Surface::Evaluate within the tolerances of the reference's own Bfr-versus-Far
regression (regression/bfr_evaluate/main.cpp:610-830).
"""
import glob
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MESHES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "bfr_*.npz"))
                if not p.endswith(("bfr_tess_patterns.npz", "bfr_share.npz", "bfr_stencils.npz")))


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.int32)


def cases(z):
    meta, ro, rates = z["meta"], z["rate_offsets"], z["rates"]
    for i in range(len(meta)):
        reg, N, fs, pq, valid, nb, uni, _ = (int(x) for x in meta[i])
        yield i, reg, N, rates[ro[i]:ro[i + 1]], fs, pq, bool(valid), nb, bool(uni)


def test_tessellation_patterns_match_the_reference_bitwise():
    z = np.load(os.path.join(GOLDEN, "bfr_tess_patterns.npz"))
    co, fo = z["coord_offsets"], z["facet_offsets"]
    n = 0
    for i, reg, N, rates, fs, pq, valid, nb, uni in cases(z):
        ok, nc, nf, nbo, unio = oracle.tess_inventory(reg, N, rates, fs, pq)
        assert ok == valid, i
        if not valid:
            assert nc == nf == 0
            continue
        c, f = oracle.tess_generate(reg, N, rates, fs, pq)
        assert np.array_equal(bits(c.ravel()), bits(z["coords"][co[i]:co[i + 1]].ravel())), i
        assert np.array_equal(f.ravel(), z["facets"][fo[i]:fo[i + 1]]), i
        assert (nbo, unio) == (nb, uni), i
        n += 1
    assert n > 700


@pytest.mark.parametrize("path", MESHES, ids=os.path.basename)
def test_mesh_tessellation_and_location_match_bfr(path):
    z = np.load(path)
    reg = int(z["regular_face_size"])
    sizes = z["verts_per_face"]
    t = oracle.tess_mesh(reg, sizes, z["rate_offsets"], z["rates"], int(z["facet_size"]),
                         bool(z["preserve_quads"]), threads=4)
    assert np.array_equal(t["coord_offsets"], z["coord_offsets"])
    assert np.array_equal(t["facet_offsets"] * t["facets"].shape[1], z["facet_offsets"] *
                          z["facets"].shape[1])
    assert np.array_equal(bits(t["coords"]), bits(z["coords"]))
    assert np.array_equal(t["facets"], z["facets"])
    # sub-face conversion and ptex numbering of every coord
    co = z["coord_offsets"]
    faces, st = [], []
    for f in range(len(sizes)):
        if co[f + 1] == co[f]:
            continue
        sub, s = oracle.param_to_subface(reg, int(sizes[f]), z["coords"][co[f]:co[f + 1]])
        faces.append(z["ptex_offsets"][f] + sub)
        st.append(s)
    faces = np.concatenate(faces).astype(np.int32)
    st = np.concatenate(st)
    assert np.array_equal(faces, z["q_face"])
    assert np.array_equal(bits(st[:, 0]), bits(z["q_s"]))
    assert np.array_equal(bits(st[:, 1]), bits(z["q_t"]))
    pm = oracle.PatchMap(z["arrays"], z["params"], bool(z["triangular"]))
    h = pm.find(faces, st[:, 0].astype(np.float64), st[:, 1].astype(np.float64))
    assert np.array_equal(h, z["q_handles"])
    assert z["q_found"].all()


def bfr_tolerances(positions):
    """The reference's Bfr-versus-Far regression tolerances (regression/bfr_evaluate/
    main.cpp:536-563, 676-690): positions within 5e-5 of the largest bounding-box extent,
    first derivatives within 5 times that, second derivatives within 25 times."""
    p = np.asarray(positions, np.float64).reshape(-1, 3)
    ptol = 5e-5 * float((p.max(0) - p.min(0)).max())
    return (ptol, 5 * ptol, 5 * ptol, 25 * ptol, 25 * ptol, 25 * ptol)


def rotated_triangles(z):
    """Coords located on rotated triangle sub-patches.  Far::PatchTable::EvaluateBasis scales the
    second derivatives there by -4^depth (far/patchBasis.cpp:1339-1366: d2Scale = derivSign *
    d1Scale^2, derivSign = -1), where the parameter map s' = c - 2^depth s of a rotated triangle
    gives +4^depth.  Bfr applies the same rule inside its own patch trees, but a face Bfr
    evaluates as one regular surface has no sub-patches, so where Far's table splits such a face
    (e.g. isolating face-varying seams) the two reference paths disagree in the sign of the
    second derivatives.  The device reproduces Far (EvalPatches' contract)."""
    prm = z["params"][z["q_handles"][:, 1]]
    arr = z["arrays"][z["q_handles"][:, 0]]
    regular = (prm[:, 1] >> 5) & 1
    ptype = np.where(regular == 1, arr[:, 0], arr[:, 1])
    depth = prm[:, 1] & 0xF
    u, v = (prm[:, 1] >> 22) & 0x3FF, (prm[:, 1] >> 12) & 0x3FF
    return np.isin(ptype, (4, 5, 10)) & ((u + v) >= (1 << depth))


def second_derivative_error(far, bfr, flip):
    """|far - bfr|, with the sign of Far's value taken back on the points in `flip`."""
    far = np.array(far, np.float64)
    far[flip] = -far[flip]
    return np.abs(far - bfr)


@pytest.mark.parametrize("path", MESHES, ids=os.path.basename)
def test_far_table_evaluation_agrees_with_bfr_surfaces(path):
    """The Far table at the located coords (the oracle's EvalPatches, float) against
    Bfr::Surface::Evaluate (float) within the reference's own Bfr-versus-Far tolerances."""
    z = np.load(path)
    coords = oracle.make_coords(z["q_handles"], z["q_s"], z["q_t"])
    n = len(coords)
    outs = [np.zeros(n * 3, np.float32) for _ in range(6)]
    assert oracle.eval_patches(z["src"], (0, 3, 3), outs, [(0, 3, 3)] * 6, coords, z["arrays"],
                               z["patch_indices"], z["params"], threads=4)
    tol = bfr_tolerances(z["positions"])
    rot = rotated_triangles(z)
    for k in range(6):
        far = outs[k].reshape(-1, 3).astype(np.float64)
        if k < 3:
            assert np.abs(far - z["out6"][k]).max() <= tol[k], k
        else:
            # where Bfr's surface is not split the sign differs on rotated sub-triangles (above)
            err = np.minimum(np.abs(far - z["out6"][k]),
                             second_derivative_error(far, z["out6"][k], rot))
            assert err.max() <= tol[k], k


def test_param_conversion_against_the_reference_library():
    """Direct comparison with the reference's Bfr::Parameterization where it is built here."""
    import ref
    if not ref.available():
        pytest.skip("reference library not built")
    rng = np.random.default_rng(5)
    for N in (3, 5, 6, 7, 9, 10, 12, 17, 40):
        uv = np.concatenate([oracle.tess_generate(4, N, [7])[0],
                             (rng.random((300, 2)) * 4).astype(np.float32)])
        a = ref.bfr_subface(4, N, uv)
        b = oracle.param_to_subface(4, N, uv)
        assert np.array_equal(a[0], b[0]) and np.array_equal(bits(a[1]), bits(b[1])), N


UV_MESHES = [p for p in MESHES if "_uv_" in os.path.basename(p)]


@pytest.mark.parametrize("path", UV_MESHES, ids=os.path.basename)
def test_far_face_varying_patches_agree_with_bfr_uv_surfaces(path):
    """Face-varying channel 0 (UVs with seams): the Far table's face-varying patches at the
    located coords against Bfr's face-varying surfaces (SurfaceFactory::InitFaceVaryingSurface,
    the reference's tutorial 1.3), within the UV tolerance of the reference's Bfr regression
    (regression/bfr_evaluate/main.cpp:123-125: 1e-4), derivatives within 5 times that."""
    z = np.load(path)
    coords = oracle.make_coords(z["q_handles"], z["q_s"], z["q_t"])
    n = len(coords)
    outs = [np.zeros(n * 2, np.float32) for _ in range(3)]
    assert oracle.eval_patches(z["fvar_src"], (0, 2, 2), outs, [(0, 2, 2)] * 3, coords,
                               z["fvar_arrays"], z["fvar_indices"], z["fvar_params"], threads=4)
    for k, tol in enumerate((1e-4, 5e-4, 5e-4)):
        assert np.abs(outs[k].reshape(-1, 2) - z["uv3"][k]).max() <= tol, k


SHARE = os.path.join(GOLDEN, "bfr_share.npz")


def share_inputs(z):
    """(face edges per corner, number of edges) for a mesh fixture: the oracle's own edge
    numbering (shared points do not depend on how edges are numbered)."""
    return oracle.edge_numbering(z["verts_per_face"], z["face_verts"])


@pytest.mark.parametrize("path", MESHES, ids=os.path.basename)
def test_shared_points_match_the_reference_tutorial(path):
    """The shared-point bookkeeping (tutorial 2.2's, restated in oracle/bfr_oracle.c) against
    the reference's own Tessellation + TransformFacetCoordIndices run through that loop
    (tests/golden/bfr_share.npz): facets as point indices, each face's first point, and the
    coord every point is evaluated at -- exactly; and every facet corner of a point lies where
    that point's source coord lies (the two faces' coords name the same surface point)."""
    z = np.load(path)
    g = np.load(SHARE)
    key = os.path.basename(path)[:-4]
    fe, ne = share_inputs(z)
    facets, po, src = oracle.tess_share(
        int(z["regular_face_size"]), z["verts_per_face"], z["face_verts"], fe,
        len(z["positions"]), ne, z["rate_offsets"], z["rates"], z["coord_offsets"],
        z["facet_offsets"], z["facets"], int(z["facet_size"]), bool(z["preserve_quads"]))
    assert np.array_equal(facets, g[key + "__facets"])
    assert np.array_equal(po, g[key + "__point_offsets"])
    assert np.array_equal(src, g[key + "__point_sources"])
    # every point is used, and every coord maps to a point evaluated within the Bfr tolerance
    fs = int(z["facet_size"])
    used = np.zeros(len(src), bool)
    used[facets[facets >= 0]] = True
    assert used.all()
    coord_of = z["facets"].reshape(-1, fs)
    m = coord_of >= 0
    p_coord = z["out6"][0][coord_of[m]]
    p_point = z["out6"][0][src[facets[m]]]
    ptol = bfr_tolerances(z["positions"])[0]
    assert np.abs(p_coord - p_point).max() <= ptol


def test_shared_points_reject_edges_with_two_rates():
    """An edge run at two rates by its two faces cannot share its points: rejected (a face's
    edge rates from edge lengths are always consistent)."""
    sizes = np.array([4, 4], np.int32)
    fv = np.array([0, 1, 4, 3, 1, 2, 5, 4], np.int32)
    fe, ne = oracle.edge_numbering(sizes, fv)
    ro = np.array([0, 4, 8], np.int32)
    rates = np.array([2, 3, 2, 3, 2, 3, 2, 4], np.int32)  # shared edge 1-4: 3 vs 4
    mesh = oracle.tess_mesh(4, sizes, ro, rates)
    with pytest.raises(ValueError):
        oracle.tess_share(4, sizes, fv, fe, 6, ne, ro, rates, mesh["coord_offsets"],
                          mesh["facet_offsets"], mesh["facets"])


STENCILS = os.path.join(GOLDEN, "bfr_stencils.npz")
STENCIL_MESHES = sorted({k.split("__")[0] for k in np.load(STENCILS).files})


def point_base(z, g, key):
    """Stencils of every point the fixture's patch indices name: identity rows for the cage
    vertices, then Far's stencils of the refined and local points (the fixture's source rows)."""
    nc = len(z["positions"])
    st = {k: g[f"{key}__st_{k}"] for k in ("sizes", "offsets", "indices", "weights")}
    return dict(sizes=np.concatenate([np.ones(nc, np.int32), st["sizes"]]).astype(np.int32),
                offsets=np.concatenate([np.arange(nc), nc + st["offsets"]]).astype(np.int32),
                indices=np.concatenate([np.arange(nc), st["indices"]]).astype(np.int32),
                weights=np.concatenate([np.ones(nc, np.float32), st["weights"]]))


def apply_stencils(sizes, indices, weights, points):
    """sum_j w_j x_j per stencil, in double."""
    rows = np.repeat(np.arange(len(sizes)), sizes)
    out = np.zeros((len(sizes), points.shape[1]))
    np.add.at(out, rows, weights.astype(np.float64)[:, None] * points[indices])
    return out


def oracle_point_stencils(z, base, channels=3):
    coords = oracle.make_coords(z["q_handles"], z["q_s"], z["q_t"])
    off, src, ws = oracle.patch_masks(coords, z["arrays"], z["patch_indices"], z["params"],
                                      channels)
    return oracle.compose_rows(base, off, src, ws)


@pytest.mark.parametrize("key", STENCIL_MESHES)
def test_point_stencils_match_bfr_evaluate_stencil(key):
    """Limit stencils at every tessellation coord over the cage vertices -- the patch basis of
    the coord's Far patch merged over the stencils of the patch's points, as
    Far::LimitStencilTableFactory merges them -- against the reference's
    Bfr::Surface::EvaluateStencil at the same coords (tests/golden/bfr_stencils.npz): applied
    to the cage, within the reference's Bfr-versus-Far tolerances; and on faces Bfr evaluates
    as regular patches, weight for weight (both are the B-spline weights of the same 16
    points)."""
    z = np.load(os.path.join(GOLDEN, key + ".npz"))
    g = np.load(STENCILS)
    ours = oracle_point_stencils(z, point_base(z, g, key))
    pos = z["positions"].astype(np.float64)
    bs = g[f"{key}__bfr_sizes"]
    bi = g[f"{key}__bfr_indices"]
    tol = bfr_tolerances(z["positions"])
    rot = rotated_triangles(z)
    for k, (ow, bw) in enumerate((("weights", "wP"), ("du_weights", "wDu"),
                                  ("dv_weights", "wDv"))):
        a = apply_stencils(ours["sizes"], ours["indices"], ours[ow], pos)
        b = apply_stencils(bs, bi, g[f"{key}__bfr_{bw}"], pos)
        assert np.abs(a - b).max() <= tol[k], (key, k, np.abs(a - b).max(), tol[k])
        assert np.abs(a - z["out6"][k]).max() <= tol[k], k
    # regular faces: dense weights
    nc = len(pos)
    co = z["coord_offsets"]
    regular = np.repeat(z["regular"] == 1, np.diff(co))
    ob = np.concatenate([[0], np.cumsum(ours["sizes"])])
    bb = np.concatenate([[0], np.cumsum(bs)])
    checked = 0
    for i in np.nonzero(regular)[0][::7]:
        for ow, bw in (("weights", "wP"), ("du_weights", "wDu"), ("dv_weights", "wDv")):
            da = np.zeros(nc)
            np.add.at(da, ours["indices"][ob[i]:ob[i + 1]], ours[ow][ob[i]:ob[i + 1]])
            db = np.zeros(nc)
            np.add.at(db, bi[bb[i]:bb[i + 1]], g[f"{key}__bfr_{bw}"][bb[i]:bb[i + 1]])
            assert np.abs(da - db).max() <= 2e-6 * max(1.0, np.abs(db).max()), (key, i, ow)
        checked += 1
    assert checked > 0 or not regular.any()


def varying_source(g, key):
    """Varying values of the control vertices, then of every refined vertex (Far's varying
    stencils): the points the varying patches index."""
    vals = g[f"{key}__var_values"]
    nc = len(vals)
    sizes = g[f"{key}__var_st_sizes"]
    src = np.zeros((nc + len(sizes)) * 3, np.float32)
    src[: nc * 3] = vals.ravel()
    oracle.eval_stencils(src, (0, 3, 3), [src], [(nc * 3, 3, 3)], sizes,
                         g[f"{key}__var_st_offsets"], g[f"{key}__var_st_indices"],
                         [g[f"{key}__var_st_weights"]])
    return src


@pytest.mark.parametrize("key", STENCIL_MESHES)
def test_far_varying_patches_agree_with_bfr_varying_surfaces(key):
    """Bfr::SurfaceFactory::InitVaryingSurface evaluated by the reference at every coord
    against the paired Far table's varying patches at the located coords, over Far's varying
    refinement of the same values: equal within float rounding (1e-6)."""
    z = np.load(os.path.join(GOLDEN, key + ".npz"))
    g = np.load(STENCILS)
    src = varying_source(g, key)
    coords = oracle.make_coords(z["q_handles"], z["q_s"], z["q_t"])
    out = [np.zeros(len(coords) * 3, np.float32)]
    assert oracle.eval_patches(src, (0, 3, 3), out, [(0, 3, 3)], coords, g[f"{key}__var_arrays"],
                               g[f"{key}__var_indices"], z["params"], threads=4)
    assert np.abs(out[0].reshape(-1, 3) - g[f"{key}__var_bfr"]).max() <= 1e-6


@pytest.mark.parametrize("key", STENCIL_MESHES)
def test_limit_option_rates_agree_with_tutorial_2_1(key):
    """Tutorial 2.1's limit option (rates from the limit positions at each face's corners,
    computed by the reference's Bfr in tests/golden/bfr_stencils.npz) against the same rule on
    the paired Far table's limit positions at the located corner coords: the corner points
    within the Bfr-vs-Far position tolerance, and the rates equal wherever the length quotient
    is not within that tolerance of an integer (where either side may round across it)."""
    from opensubdiv_gb300.bfr import Parameterization
    z = np.load(os.path.join(GOLDEN, key + ".npz"))
    g = np.load(STENCILS)
    reg = int(z["regular_face_size"])
    sizes = z["verts_per_face"]
    want, want_pts = g[f"{key}__limit_rates"], g[f"{key}__limit_points"]
    pos = z["positions"]
    ext = float((pos.max(0) - pos.min(0)).max())
    interval, max_rate = ext / 40.0, 10
    ptex = z["ptex_offsets"]
    faces, sts, corners = [], [], []
    start = np.concatenate([[0], np.cumsum(sizes)])
    for f in range(len(sizes)):
        if want[start[f]] == 0:
            continue
        N = int(sizes[f])
        uv = np.array([Parameterization(reg, N).GetVertexCoord(i) for i in range(N)], np.float32)
        sub, st = oracle.param_to_subface(reg, N, uv)
        faces.append(ptex[f] + sub)
        sts.append(st)
        corners.append(np.arange(start[f], start[f] + N))
    faces, sts, corners = np.concatenate(faces), np.concatenate(sts), np.concatenate(corners)
    pm = oracle.PatchMap(z["arrays"], z["params"], bool(z["triangular"]))
    h = pm.find(faces, sts[:, 0].astype(np.float64), sts[:, 1].astype(np.float64))
    coords = oracle.make_coords(h, sts[:, 0], sts[:, 1])
    P = [np.zeros(len(coords) * 3, np.float32)]
    assert oracle.eval_patches(z["src"], (0, 3, 3), P, [(0, 3, 3)], coords, z["arrays"],
                               z["patch_indices"], z["params"], threads=4)
    P = P[0].reshape(-1, 3)
    ptol = 5e-5 * ext
    assert np.abs(P - want_pts[corners]).max() <= ptol
    # the rule on the Far points, per face (corner i to corner i + 1 of the same face)
    got = np.zeros_like(want)
    quotient = np.zeros(len(want))
    k = 0
    for f in range(len(sizes)):
        if want[start[f]] == 0:
            continue
        N = int(sizes[f])
        pts = P[k:k + N]
        k += N
        d = np.abs(pts - np.roll(pts, -1, axis=0))
        length = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
        q = length / np.float32(interval)
        got[start[f]:start[f] + N] = np.minimum(1 + q.astype(np.int32), max_rate)
        quotient[start[f]:start[f] + N] = q
    near = np.abs(quotient - np.round(quotient)) <= 2 * ptol / interval
    assert np.array_equal(got[~near], want[~near])
    assert np.all(np.abs(got[near] - want[near]) <= 1)
