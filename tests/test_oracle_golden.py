"""Pin the C oracle (oracle/osd_oracle.c) to the reference's own outputs.

The fixtures in tests/golden/ were produced by the reference (Far factories, Osd::CpuEvaluator,
Far::PatchMap, Far::PatchTable::EvaluateBasis<double>) through tests/golden/make_golden.py.
The oracle must reproduce the float results bit for bit, the PatchMap handles exactly and the
FP64 results exactly.
"""
import glob
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STENCIL_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "*_uniform_L*.npz")))
PATCH_FIXTURES = sorted(set(glob.glob(os.path.join(GOLDEN, "*_patches_*.npz"))) |
                        set(glob.glob(os.path.join(GOLDEN, "*_uniform_quads_*.npz"))) |
                        set(glob.glob(os.path.join(GOLDEN, "*_uniform_tris_*.npz"))))


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.int32)


@pytest.mark.parametrize("path", STENCIL_FIXTURES, ids=os.path.basename)
def test_eval_stencils_bitwise(path):
    z = np.load(path)
    n = len(z["sizes"])
    tbl = (z["sizes"], z["offsets"], z["indices"])
    o3 = np.zeros(n * 3, np.float32)
    assert oracle.eval_stencils(z["positions"].ravel(), (0, 3, 3), [o3], [(0, 3, 3)], *tbl,
                                [z["weights"]])
    assert np.array_equal(bits(o3), bits(z["out3"]))
    o8 = np.zeros(n * 8, np.float32)
    assert oracle.eval_stencils(z["src8"], (0, 8, 8), [o8], [(0, 8, 8)], *tbl, [z["weights"]])
    assert np.array_equal(bits(o8), bits(z["out8"]))
    o5 = np.zeros(n * 5 + 5, np.float32)
    assert oracle.eval_stencils(z["src7"], (2, 3, 7), [o5], [(1, 3, 5)], *tbl, [z["weights"]])
    assert np.array_equal(bits(o5), bits(z["out_strided"]))
    # in place: source and destination are one buffer (osd/mesh.h:501-540)
    nc = len(z["positions"])
    buf = np.zeros((nc + n) * 3, np.float32)
    buf[: nc * 3] = z["positions"].ravel()
    assert oracle.eval_stencils(buf, (0, 3, 3), [buf], [(nc * 3, 3, 3)], *tbl, [z["weights"]])
    assert np.array_equal(bits(buf), bits(z["out_inplace"]))


@pytest.mark.parametrize("path", [p for p in STENCIL_FIXTURES if "limit_sizes" in np.load(p)],
                         ids=os.path.basename)
def test_eval_limit_stencils_with_derivatives_bitwise(path):
    z = np.load(path)
    m = len(z["limit_sizes"])
    names = ("weights", "du_weights", "dv_weights", "duu_weights", "duv_weights", "dvv_weights")
    ws = [z["limit_" + k] for k in names]
    tbl = (z["limit_sizes"], z["limit_offsets"], z["limit_indices"])
    for nout in (1, 3, 6):
        outs = [np.zeros(m * 3, np.float32) for _ in range(nout)]
        assert oracle.eval_stencils(z["positions"].ravel(), (0, 3, 3), outs, [(0, 3, 3)] * nout,
                                    *tbl, ws[:nout])
        for k in range(nout):
            assert np.array_equal(bits(outs[k]), bits(z["limit_out6"][k])), names[k]


@pytest.mark.parametrize("path", STENCIL_FIXTURES, ids=os.path.basename)
def test_fp64_stencils_against_reference_double_tables(path):
    """The FP64 oracle (float tables applied in double) against the reference's double
    factory (same indices, double weights): they differ only by the float rounding of the
    weights."""
    z = np.load(path)
    n = len(z["sizes"])
    od = np.zeros(n * 3, np.float64)
    assert oracle.eval_stencils(z["positions"].ravel(), (0, 3, 3), [od], [(0, 3, 3)], z["sizes"],
                                z["offsets"], z["indices"], [z["weights"]], fp64=True)
    src = z["positions"].astype(np.float64)
    rows = np.repeat(np.arange(n), z["sizes"])
    ref64 = np.zeros((n, 3))
    np.add.at(ref64, rows, z["weights_fp64"][:, None] * src[z["indices"]])
    diag = float(np.linalg.norm(src.max(0) - src.min(0)))
    assert np.abs(od.reshape(n, 3) - ref64).max() <= 1e-6 * diag
    # and the float result is within the accuracy bound of both
    assert np.abs(z["out3"].reshape(n, 3) - ref64).max() <= 1e-5 * diag


@pytest.mark.parametrize("path", PATCH_FIXTURES, ids=os.path.basename)
def test_patchmap_handles_exact(path):
    z = np.load(path)
    pm = oracle.PatchMap(z["arrays"], z["params"], int(z["triangular"]))
    h = pm.find(z["q_face"], z["q_u"].astype(np.float64), z["q_v"].astype(np.float64))
    assert np.array_equal(h, z["q_handles"])
    assert np.array_equal((h[:, 0] >= 0).astype(np.int32), z["q_found"])


@pytest.mark.parametrize("path", PATCH_FIXTURES, ids=os.path.basename)
def test_eval_patches_bitwise_and_fp64(path):
    z = np.load(path)
    m = z["coords"].shape[0]
    args = (z["coords"], z["arrays"], z["patch_indices"], z["params"])
    outs = [np.zeros(m * 3, np.float32) for _ in range(6)]
    assert oracle.eval_patches(z["src"], (0, 3, 3), outs, [(0, 3, 3)] * 6, *args)
    for k in range(6):
        assert np.array_equal(bits(outs[k]), bits(z["out6"][k].ravel())), k
    outd = [np.zeros(m * 3, np.float64) for _ in range(6)]
    assert oracle.eval_patches(z["src"], (0, 3, 3), outd, [(0, 3, 3)] * 6, *args, fp64=True)
    for k in range(6):
        assert np.array_equal(outd[k], z["out6_fp64"][k].ravel()), k


@pytest.mark.parametrize("path", PATCH_FIXTURES, ids=os.path.basename)
def test_patch_point_stencils_reproduce_the_patch_source(path):
    """The patch points' stencils over the cage (stored with each patch fixture) reproduce the
    patch source the reference computed in place: src[nc:] = stencils applied to src[:nc]."""
    z = np.load(path)
    nc = len(z["positions"])
    n = len(z["ps_sizes"])
    assert len(z["src"]) == 3 * (nc + n)
    assert n == 0 or int(z["ps_indices"].max()) < nc  # factorized to the cage
    out = np.zeros(n * 3, np.float32)
    oracle.eval_stencils(z["src"][: nc * 3], (0, 3, 3), [out], [(0, 3, 3)], z["ps_sizes"],
                         z["ps_offsets"], z["ps_indices"], [z["ps_weights"]])
    assert np.array_equal(out, z["src"][nc * 3:])


FVAR_FIXTURES = [p for p in PATCH_FIXTURES if "fvar_arrays" in np.load(p)]


@pytest.mark.parametrize("path", FVAR_FIXTURES, ids=os.path.basename)
def test_varying_and_face_varying_patches_bitwise(path):
    """EvalPatchesVarying (vertex params with the varying arrays/indices) and
    EvalPatchesFaceVarying (the channel's own arrays/indices/params) restated, against
    Osd::CpuEvaluator on the reference's own varying / face-varying tables."""
    z = np.load(path)
    m = z["coords"].shape[0]
    vo = [np.zeros(m * 4, np.float32) for _ in range(3)]
    oracle.eval_patches(z["varying_src"], (0, 4, 4), vo, [(0, 4, 4)] * 3, z["coords"],
                        z["varying_arrays"], z["varying_indices"], z["params"])
    for k in range(3):
        assert np.array_equal(vo[k], z["varying_out3"][k].ravel()), k
    fo = [np.zeros(m * 2, np.float32) for _ in range(6)]
    oracle.eval_patches(z["fvar_src"], (0, 2, 2), fo, [(0, 2, 2)] * 6, z["coords"],
                        z["fvar_arrays"], z["fvar_indices"], z["fvar_params"])
    for k in range(6):
        assert np.array_equal(fo[k], z["fvar_out6"][k].ravel()), k


def test_descriptor_length_mismatch_is_rejected():
    """CpuEvaluator returns false when a destination length differs from the source's
    (osd/cpuEvaluator.cpp:46-47)."""
    z = np.load(STENCIL_FIXTURES[0])
    o = np.zeros(len(z["sizes"]) * 4, np.float32)
    assert not oracle.eval_stencils(z["positions"].ravel(), (0, 3, 3), [o], [(0, 4, 4)],
                                    z["sizes"], z["offsets"], z["indices"], [z["weights"]])
