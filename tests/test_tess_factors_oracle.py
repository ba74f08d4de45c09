"""The oracle's restatement of the patch shaders' tessellation-factor math
(osd/glslPatchCommonTess.glsl): the properties the shader source states, checked on the CPU."""
import os

import numpy as np

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_uniform_levels_halve_per_refinement_level_and_clamp_transitions():
    """OsdGetTessLevelsUniform: min(level, max) / 2^(depth - 1), at least 2 on transition edges
    and 1 elsewhere; inner levels are the averages of opposite outer levels (equal spacing)."""
    z = np.load(os.path.join(GOLDEN, "torus32x16_patches_L4.npz"))
    params = z["params"]
    depth = params[:, 1] & 0xF
    trans = (params[:, 0] >> 28) & 0xF
    outer, inner, lo, hi = oracle.tess_factors(z["arrays"], z["patch_indices"], params, None, 3,
                                               6.0, 64.0, False, 0)
    base = 6.0 / 2.0 ** (depth - 1)
    for e, bit in enumerate((8, 1, 2, 4)):
        mn = 1 + ((trans & bit) != 0)
        assert np.array_equal(outer[:, e], np.round(np.maximum(base, mn)).astype(np.float32))
    assert (hi == 0).all()
    assert np.allclose(inner[:, 0], (outer[:, 1] + outer[:, 3]) / 2)
    assert np.allclose(inner[:, 1], (outer[:, 0] + outer[:, 2]) / 2)


def test_transition_parameterization_maps_the_edge_onto_two_halves():
    """OsdGetTessTransitionSplit, equal spacing: domain points along a split edge land on its
    two halves, the first lo segments on [0, 1/2] and the rest on [1/2, 1], endpoints fixed."""
    lo = np.array([[3, 0, 0, 0]], np.float32)
    hi = np.array([[5, 0, 0, 0]], np.float32)
    t = np.arange(9, dtype=np.float32) / 8
    d = np.stack([np.zeros(9), t, np.zeros(9)], 1).astype(np.float32)
    uv = oracle.tess_parameterization(d, np.zeros(9, np.int32), lo, hi, 0, False)
    assert np.allclose(uv[:, 0], 0)
    assert np.allclose(uv[:4, 1], np.arange(4) / 3 * 0.5)
    assert np.allclose(uv[3:, 1], 0.5 + np.arange(6) / 5 * 0.5)
