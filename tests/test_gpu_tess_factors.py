"""Draw-time tessellation factors of the patch shaders (GB300PatchTableTessFactors,
GB300PatchTessParameterization) against the oracle's restatement of
osd/glslPatchCommonTess.glsl, on the reference's adaptive tables (transition edges, Gregory-basis
end caps, boundaries; Loop tables with Gregory triangles).

The reference's version is GLSL, which cannot run without a graphics stack, so the restatement
is read from the shader source and not pinned against an execution of it.  Uniform factors are
integer / power-of-two arithmetic and must match exactly; screen-space factors come from limit
positions the GPU and the oracle evaluate with different summation orders, so the unrounded
levels are compared within 1e-4 relative and the rounded ones exactly except where the
unrounded level sits within 1e-3 of a rounding boundary.
"""
import os

import numpy as np
import pytest

import oracle
from gpu_util import dev, host, torch_cuda

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TABLES = ["torus32x16_patches_L4.npz", "icosphere2_patches_L3.npz", "grid6_patches_L3.npz",
          "trigrid6_patches_L3.npz"]


def look_at(eye, target, up):
    f = np.asarray(target, np.float64) - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m


def perspective(fovy, aspect, near, far):
    f = 1.0 / np.tan(fovy / 2)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = f / aspect, f
    m[2, 2], m[2, 3] = (far + near) / (near - far), 2 * far * near / (near - far)
    m[3, 2] = -1.0
    return m


def camera(positions):
    p = np.asarray(positions, np.float64)
    c = 0.5 * (p.min(0) + p.max(0))
    r = np.linalg.norm(p.max(0) - p.min(0))
    return look_at(c + np.array([0.3, 0.4, 1.0]) * r, c, np.array([0.0, 1.0, 0.0])), \
        perspective(np.radians(45.0), 1.0, 0.01 * r, 10.0 * r)


def run_gpu(z, opts, src):
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import GB300PatchTable
    t = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"],
                               bool(z["triangular"]))
    n = len(z["params"])
    outs = [torch.zeros((n, 4), device="cuda"), torch.zeros((n, 2), device="cuda"),
            torch.zeros((n, 4), device="cuda"), torch.zeros((n, 4), device="cuda")]
    t.TessFactors(opts, outs[0], outs[1], outs[2], outs[3], src=dev(src) if src is not None
                  else None, src_stride=3)
    torch.cuda.synchronize()
    return [host(o) for o in outs]


@pytest.mark.gpu
@pytest.mark.parametrize("name", TABLES)
def test_uniform_factors_exact(name):
    from opensubdiv_gb300.evaluator import PatchTessOptions
    z = np.load(os.path.join(GOLDEN, name))
    for level in (1.0, 3.0, 8.0, 16.0, 64.0):
        for spacing in (0, 1, 2):
            got = run_gpu(z, PatchTessOptions(level, 64.0, False, spacing), None)
            want = oracle.tess_factors(z["arrays"], z["patch_indices"], z["params"], None, 3,
                                       level, 64.0, False, spacing)
            for g, w in zip(got, want):
                assert np.array_equal(g, w), (level, spacing)


@pytest.mark.gpu
@pytest.mark.parametrize("name", TABLES)
@pytest.mark.parametrize("spacing", [0, 1, 2])
def test_screen_space_factors(name, spacing):
    from opensubdiv_gb300.evaluator import PatchTessOptions
    z = np.load(os.path.join(GOLDEN, name))
    mv, pr = camera(z["positions"])
    opts = PatchTessOptions(24.0, 64.0, True, spacing, mv, pr)
    got = run_gpu(z, opts, z["src"])
    want = oracle.tess_factors(z["arrays"], z["patch_indices"], z["params"], z["src"], 3, 24.0,
                               64.0, True, spacing, mv, pr)
    edges = 3 if int(z["triangular"]) else 4
    assert (want[0][:, :edges] >= 1).all()
    # fractional spacings keep the unrounded halves: compare them directly
    if spacing != 0:
        for g, w in zip(got[2:], want[2:]):
            assert np.allclose(g, w, rtol=1e-4, atol=1e-5)
    # rounded levels: equal except where a level next to a rounding boundary went the other
    # way (one rounding step: 1 for equal spacing, 2 for the even / odd round-ups)
    mismatch = ~np.isclose(got[0], want[0], rtol=1e-4, atol=1e-4)
    assert mismatch.mean() < 1e-3, mismatch.mean()
    assert np.abs(got[0] - want[0])[mismatch].max(initial=0.0) <= 2.0 + 1e-3
    assert np.allclose(got[1], want[1], rtol=1e-4, atol=1.0 + 1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("spacing", [0, 1, 2])
def test_transition_parameterization(spacing):
    torch = torch_cuda()
    from opensubdiv_gb300.evaluator import PatchTessOptions, PatchTessParameterization
    z = np.load(os.path.join(GOLDEN, "torus32x16_patches_L4.npz"))
    mv, pr = camera(z["positions"])
    opts = PatchTessOptions(24.0, 64.0, True, spacing, mv, pr)
    outer, inner, lo, hi = oracle.tess_factors(z["arrays"], z["patch_indices"], z["params"],
                                               z["src"], 3, 24.0, 64.0, True, spacing, mv, pr)
    split = np.nonzero((hi > 0).any(1))[0]
    assert len(split) > 0
    rng = np.random.default_rng(spacing)
    pts, pid = [], []
    for p in split[:400]:
        for e in range(4):
            t = np.linspace(0.0, 1.0, 9)
            d = np.zeros((9, 3), np.float32)
            if e == 0:
                d[:, 1] = t
            elif e == 1:
                d[:, 0] = t
            elif e == 2:
                d[:, 0], d[:, 1] = 1.0, t
            else:
                d[:, 0], d[:, 1] = t, 1.0
            pts.append(d)
            pid += [p] * 9
    pts.append(rng.random((200, 3)).astype(np.float32))
    pid += list(rng.choice(split, 200))
    pts = np.concatenate(pts)
    pid = np.asarray(pid, np.int32)
    want = oracle.tess_parameterization(pts, pid, lo, hi, spacing, False)
    uv = torch.zeros((len(pts), 2), device="cuda")
    PatchTessParameterization(len(pts), dev(pts), dev(pid), dev(lo), dev(hi), uv, spacing)
    torch.cuda.synchronize()
    assert np.allclose(host(uv), want, atol=1e-6)
