"""EvalPatches and the device PatchMap on the GB300 through the C ABI.

Fixtures cover every patch type the Osd evaluator supports: REGULAR (B-spline, with boundary
masks on the open grid), GREGORY_BASIS end caps, LOOP (box spline, with boundary masks),
GREGORY_TRIANGLE, and the linear QUADS / TRIANGLES of uniform tables.  PatchMap handles must
be bit-exact with Far::PatchMap (integer work).  Float outputs pass the accuracy gate of
tests/gpu_util.py (`gate`) at 1e-5 x the bounding-box diagonal with no scaling: P, dPdu and
dPdv against Osd::CpuEvaluator, the second derivatives against the FP64 evaluation.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from gpu_util import bbox_diag, bbox_diag_rows, dev, gate, host, smooth_primvars, torch_cuda

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(set(glob.glob(os.path.join(GOLDEN, "*_patches_*.npz"))) |
                  set(glob.glob(os.path.join(GOLDEN, "*_uniform_quads_*.npz"))) |
                  set(glob.glob(os.path.join(GOLDEN, "*_uniform_tris_*.npz"))))
NAMES = ("P", "du", "dv", "duu", "duv", "dvv")


def _table(z):
    from opensubdiv_gb300.evaluator import GB300PatchTable
    return GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"],
                                  triangular=bool(z["triangular"]))


def _oracle6(src, length, coords, arrays, indices, params, fp64):
    """The six EvalPatches outputs of the oracle (CpuEvaluator, or its FP64 form)."""
    m = coords.shape[0]
    outs = [np.zeros(m * length, np.float64 if fp64 else np.float32) for _ in range(6)]
    oracle.eval_patches(src, (0, length, length), outs, [(0, length, length)] * 6, coords,
                        arrays, indices, params, threads=8, fp64=fp64)
    return outs


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_device_patchmap_bit_exact(path):
    torch = torch_cuda()
    z = np.load(path)
    t = _table(z)
    n = len(z["q_face"])
    out = torch.zeros(n * 5, dtype=torch.int32, device="cuda")
    t.FindPatches(n, dev(z["q_face"]), dev(z["q_u"]), dev(z["q_v"]), out)
    torch.cuda.synchronize()
    o = host(out).reshape(n, 5)
    assert np.array_equal(o[:, :3], z["q_handles"])
    assert np.array_equal(o[:, 3].view(np.float32), z["q_u"])
    assert np.array_equal(o[:, 4].view(np.float32), z["q_v"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_eval_patches_all_outputs(path):
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300Evaluator as Ev
    z = np.load(path)
    m = z["coords"].shape[0]
    t = _table(z)
    src = dev(z["src"])
    coords = dev(z["coords"])
    outs = [torch.zeros(m * 3, device="cuda") for _ in range(6)]
    d = BD(0, 3, 3)
    assert Ev.EvalPatchesTable(src, d, outs[0], d, m, coords, t, du=outs[1], duDesc=d,
                               dv=outs[2], dvDesc=d, duu=outs[3], duuDesc=d, duv=outs[4],
                               duvDesc=d, dvv=outs[5], dvvDesc=d)
    Ev.Synchronize()
    diag = bbox_diag(z["positions"])
    for k in range(6):
        gate(os.path.basename(path)[:-4], k, host(outs[k]), z["out6"][k].ravel(),
             z["out6_fp64"][k].ravel(), diag)


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_eval_patches_raw_api_and_partial_outputs(path):
    """Raw-pointer API (CudaEvalPatches / ...WithDerivatives) with 1 and 3 outputs, and an
    interleaved 8-wide source evaluated at descriptor offsets."""
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300Evaluator as Ev
    z = np.load(path)
    m = z["coords"].shape[0]
    t = _table(z)
    arrays, idx, params = (t.GetPatchArrayBuffer(), t.GetPatchIndexBuffer(),
                           t.GetPatchParamBuffer())
    coords = dev(z["coords"])
    src = dev(z["src"])
    p = torch.zeros(m * 3, device="cuda")
    assert Ev.EvalPatches(src, BD(0, 3, 3), p, BD(0, 3, 3), m, coords, arrays, idx, params)
    Ev.Synchronize()
    name = os.path.basename(path)[:-4]
    diag = bbox_diag(z["positions"])
    gate(name + " raw P", 0, host(p), z["out6"][0].ravel(), None, diag)
    # 8 interleaved primvars: xyz in lanes 2..4 of a stride-8 source (smooth functions of
    # position in the other lanes), outputs stride 4
    s8 = smooth_primvars(z["src"].reshape(-1, 3))
    d = [torch.zeros(m * 4, device="cuda") for _ in range(3)]
    assert Ev.EvalPatches(dev(s8.ravel()), BD(2, 3, 8), d[0], BD(1, 3, 4), m, coords, arrays,
                          idx, params, du=d[1], duDesc=BD(0, 3, 4), dv=d[2], dvDesc=BD(1, 3, 4))
    Ev.Synchronize()
    o0 = host(d[0]).reshape(m, 4)[:, 1:4]
    o1 = host(d[1]).reshape(m, 4)[:, 0:3]
    o2 = host(d[2]).reshape(m, 4)[:, 1:4]
    for k, o in enumerate((o0, o1, o2)):
        gate(name + " strided", k, o, z["out6"][k], None, diag)
    # full 8-wide evaluation against the oracle
    out8 = [torch.zeros(m * 8, device="cuda") for _ in range(6)]
    b8 = BD(0, 8, 8)
    assert Ev.EvalPatches(dev(s8.ravel()), b8, out8[0], b8, m, coords, arrays, idx, params,
                          du=out8[1], duDesc=b8, dv=out8[2], dvDesc=b8, duu=out8[3],
                          duuDesc=b8, duv=out8[4], duvDesc=b8, dvv=out8[5], dvvDesc=b8)
    Ev.Synchronize()
    tab = (z["coords"], z["arrays"], z["patch_indices"], z["params"])
    ref8 = _oracle6(s8.ravel(), 8, *tab, fp64=False)
    f648 = _oracle6(s8.ravel(), 8, *tab, fp64=True)
    diag8 = bbox_diag_rows(s8, 8)
    for k in range(6):
        gate(name + " 8 primvars", k, host(out8[k]), ref8[k], f648[k], diag8)


@pytest.mark.gpu
def test_large_random_request_on_instanced_table():
    """300k random (face, u, v) on a 74k-patch table (the Gregory-basis torus fixture
    instanced 12x), including out-of-range faces: device PatchMap + EvalPatches against the
    oracle point by point."""
    torch = torch_cuda()
    from opensubdiv_gb300 import workloads
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300Evaluator as Ev
    from opensubdiv_gb300.evaluator import GB300PatchTable
    fixture = os.path.join(GOLDEN, "torus32x16_patches_L4.npz")
    arrays, indices, params, src, nptex, tri = workloads.instanced_patch_table(np.load(fixture), 12)
    assert arrays[:, 2].sum() >= 1 << 16
    t = GB300PatchTable.Create(arrays, indices, params, tri)
    n = 300_000
    rng = np.random.default_rng(3)
    face = rng.integers(-2, nptex + 2, n).astype(np.int32)  # a few misses at both ends
    u = rng.random(n).astype(np.float32)
    v = rng.random(n).astype(np.float32)
    coords = torch.zeros(n * 5, dtype=torch.int32, device="cuda")
    t.FindPatches(n, dev(face), dev(u), dev(v), coords)
    d = BD(0, 3, 3)
    outs = [torch.full((n * 3,), 9.0, device="cuda") for _ in range(6)]
    assert Ev.EvalPatchesTable(dev(src), d, outs[0], d, n, coords, t, du=outs[1], duDesc=d,
                               dv=outs[2], dvDesc=d, duu=outs[3], duuDesc=d, duv=outs[4],
                               duvDesc=d, dvv=outs[5], dvvDesc=d)
    Ev.Synchronize()
    ch = host(coords).reshape(n, 5)
    hit = ch[:, 0] >= 0
    assert 0 < (~hit).sum() < n // 100
    chh = np.ascontiguousarray(ch[hit])  # the oracle (like CpuEvaluator) takes hits only
    refs = _oracle6(src, 3, chh, arrays, indices, params, fp64=False)
    f64 = _oracle6(src, 3, chh, arrays, indices, params, fp64=True)
    # the cage is the union of the displaced copies; the reference's absolute-coordinate sums
    # lose accuracy with the distance from the origin, the local-origin gathers do not
    diag = bbox_diag_rows(src, 3)
    for k in range(6):
        g = host(outs[k]).reshape(n, 3)
        assert np.all(g[~hit] == 0)
        gate("torus32x16 x12 random 300k", k, g[hit], refs[k], f64[k], diag)


@pytest.mark.gpu
def test_patchmap_misses_evaluate_to_zero():
    """Coords with a negative array index (PatchMap misses) produce zeros."""
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300Evaluator as Ev
    z = np.load(FIXTURES[0])
    t = _table(z)
    c = z["coords"][:4].copy()
    c[1, :3] = -1
    out = torch.full((12,), 5.0, device="cuda")
    assert Ev.EvalPatchesTable(dev(z["src"]), BD(0, 3, 3), out, BD(0, 3, 3), 4, dev(c), t)
    Ev.Synchronize()
    o = host(out).reshape(4, 3)
    assert np.all(o[1] == 0)
    gate("misses", 0, o[[0, 2, 3]], z["out6"][0][[0, 2, 3]], None, bbox_diag(z["positions"]))


FVAR_FIXTURES = [p for p in FIXTURES if "fvar_arrays" in np.load(p)]


@pytest.mark.gpu
@pytest.mark.parametrize("path", FVAR_FIXTURES, ids=os.path.basename)
def test_eval_patches_varying_and_face_varying(path):
    """EvalPatchesVarying / EvalPatchesFaceVarying over the reference's varying and
    face-varying tables (non-linear face-varying patches with seams), against CpuEvaluator."""
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300Evaluator as Ev
    z = np.load(path)
    m = z["coords"].shape[0]
    t = _table(z)
    t.SetVarying(z["varying_arrays"], z["varying_indices"])
    ch = t.AddFVarChannel(z["fvar_arrays"], z["fvar_indices"], z["fvar_params"])
    assert ch == 0 and t.GetNumFVarChannels() == 1
    assert t.GetVaryingPatchIndexBuffer() and t.GetFVarPatchParamBuffer(0)
    coords = dev(z["coords"])
    # varying: 4 primvars, P + du + dv, with the vertex patch params
    d4 = BD(0, 4, 4)
    vo = [torch.zeros(m * 4, device="cuda") for _ in range(3)]
    assert Ev.EvalPatchesVarying(dev(z["varying_src"]), d4, vo[0], d4, m, coords, t, du=vo[1],
                                 duDesc=d4, dv=vo[2], dvDesc=d4)
    # face-varying: 2 primvars (uv), all six outputs
    d2 = BD(0, 2, 2)
    fo = [torch.zeros(m * 2, device="cuda") for _ in range(6)]
    assert Ev.EvalPatchesFaceVarying(dev(z["fvar_src"]), d2, fo[0], d2, m, coords, t, ch,
                                     du=fo[1], duDesc=d2, dv=fo[2], dvDesc=d2, duu=fo[3],
                                     duuDesc=d2, duv=fo[4], duvDesc=d2, dvv=fo[5], dvvDesc=d2)
    Ev.Synchronize()
    name = os.path.basename(path)[:-4]
    dv_ = bbox_diag_rows(z["varying_src"], 4)
    for k in range(3):
        gate(name + " varying", k, host(vo[k]), z["varying_out3"][k].ravel(), None, dv_)
    f64 = _oracle6(z["fvar_src"], 2, z["coords"], z["fvar_arrays"], z["fvar_indices"],
                   z["fvar_params"], fp64=True)
    df = bbox_diag_rows(z["fvar_src"], 2)
    for k in range(6):
        gate(name + " face-varying", k, host(fo[k]), z["fvar_out6"][k].ravel(), f64[k], df)
    # a varying set that does not describe the vertex patches is rejected
    from opensubdiv_gb300.evaluator import GB300Error
    bad = z["varying_arrays"].copy()
    bad[0, 2] -= 1
    with pytest.raises(GB300Error):
        t.SetVarying(bad, z["varying_indices"])
    assert not Ev.EvalPatchesFaceVarying(dev(z["fvar_src"]), d2, fo[0], d2, m, coords, t, 3)


@pytest.mark.gpu
def test_triangle_patchmap_sums_at_the_median():
    """Triangle quadtree walks decide on u + v against the median, which the reference rounds
    in double: queries whose sum lies within an ulp of a median (and sums of very different
    magnitudes) must take the reference's decisions (oracle PatchMap, pinned to Far)."""
    torch = torch_cuda()
    z = np.load(os.path.join(GOLDEN, "icosphere2_patches_L3.npz"))
    t = _table(z)
    rng = np.random.default_rng(31)
    nptex = int(z["num_ptex"])
    us, vs = [], []
    for m in (0.5, 0.25, 0.125, 0.0625):
        u = (rng.random(2000) * m).astype(np.float32)
        v = (np.float32(m) - u).astype(np.float32)
        for dv in (v, np.nextafter(v, np.float32(0)), np.nextafter(v, np.float32(1))):
            us.append(u)
            vs.append(dv)
        # one tiny operand next to a value just below the median
        us.append(np.full(500, np.nextafter(np.float32(m), np.float32(0)), np.float32))
        vs.append((rng.random(500) * 2.0 ** -40).astype(np.float32))
    # the same queries inside rotated sub-triangles (offset by the parent's median)
    u = np.concatenate(us)
    v = np.concatenate(vs)
    u2 = np.clip(np.float32(1.0) - u, 0, 1).astype(np.float32)
    v2 = np.clip(np.float32(1.0) - v, 0, 1).astype(np.float32)
    u = np.concatenate([u, np.float32(0.5) - u * np.float32(0.5), u2 * np.float32(0.5)])
    v = np.concatenate([v, np.float32(0.5) - v * np.float32(0.5), v2 * np.float32(0.5)])
    u = np.clip(u, 0, 1).astype(np.float32)
    v = np.clip(v, 0, 1).astype(np.float32)
    face = rng.integers(0, nptex, len(u)).astype(np.int32)
    n = len(face)
    out = torch.zeros(n * 5, dtype=torch.int32, device="cuda")
    t.FindPatches(n, dev(face), dev(u), dev(v), out)
    torch.cuda.synchronize()
    got = host(out).reshape(n, 5)[:, :3]
    pm = oracle.PatchMap(z["arrays"], z["params"], True)
    want = pm.find(face, u.astype(np.float64), v.astype(np.float64))
    assert np.array_equal(got, want)
