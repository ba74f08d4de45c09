"""Host-side helpers of the Bfr path, on the CPU.

* `workloads.face_edges` numbers a mesh's edges from its face vertices; the shared-point pass
  depends only on which face corners name the same edge, so it must agree with the oracle's
  own numbering and give one index per undirected edge.
* `workloads.bfr_edge_length_rates` is the rate rule of the reference's Bfr tutorial 2.1 with
  its hull option (tutorials/bfr/tutorial_2_1/bfr_tutorial_2_1.cpp:121-166): restated here as
  the tutorial's scalar loop in float, the vectorized helper must give the same rates, and the
  two faces of an edge the same rate.
* The shared-point oracle's answer does not depend on how edges are numbered.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from opensubdiv_gb300 import shapes, workloads

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MESHES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "bfr_*.npz"))
                if not p.endswith(("bfr_tess_patterns.npz", "bfr_share.npz", "bfr_stencils.npz")))


def corner_pairs(sizes, fv):
    start = np.concatenate([[0], np.cumsum(sizes)])
    for f in range(len(sizes)):
        n = int(sizes[f])
        for i in range(n):
            yield start[f] + i, int(fv[start[f] + i]), int(fv[start[f] + (i + 1) % n])


@pytest.mark.parametrize("path", MESHES, ids=os.path.basename)
def test_face_edges_name_each_undirected_edge_once(path):
    z = np.load(path)
    sizes, fv = z["verts_per_face"], z["face_verts"]
    fe, ne = workloads.face_edges(sizes, fv)
    oe, one = oracle.edge_numbering(sizes, fv)
    assert ne == one and np.array_equal(fe, oe)
    seen = {}
    for c, a, b in corner_pairs(sizes, fv):
        key = (min(a, b), max(a, b))
        assert seen.setdefault(key, fe[c]) == fe[c]
    assert len(seen) == ne and sorted(seen.values()) == list(range(ne))


def tutorial_loop_rates(pos, sizes, fv, interval, max_rate):
    """GetEdgeTessRates of tutorial 2.1 over each face's hull points, scalar float32 steps."""
    out = []
    f32 = np.float32
    for _, a, b in corner_pairs(sizes, fv):
        d = [abs(f32(pos[a][k]) - f32(pos[b][k])) for k in range(3)]
        length = np.sqrt(f32(f32(f32(d[0] * d[0]) + f32(d[1] * d[1])) + f32(d[2] * d[2])))
        out.append(min(1 + int(f32(length / f32(interval))), max_rate))
    return np.asarray(out, np.int32)


@pytest.mark.parametrize("path", MESHES[:6], ids=os.path.basename)
@pytest.mark.parametrize("divisions,max_rate", [(7.0, 10), (40.0, 10), (40.0, 64)])
def test_edge_length_rates_follow_tutorial_2_1(path, divisions, max_rate):
    z = np.load(path)
    pos, sizes, fv = z["positions"], z["verts_per_face"], z["face_verts"]
    interval = float((pos.max(0) - pos.min(0)).max()) / divisions
    off, rates = workloads.bfr_edge_length_rates(pos, sizes, fv, interval, max_rate)
    assert np.array_equal(off, np.concatenate([[0], np.cumsum(sizes)]))
    assert np.array_equal(rates, tutorial_loop_rates(pos, sizes, fv, interval, max_rate))
    fe, ne = workloads.face_edges(sizes, fv)
    per_edge = np.full(ne, -1)
    per_edge[fe] = rates
    assert np.array_equal(per_edge[fe], rates)


def test_shared_points_do_not_depend_on_edge_numbering():
    """The same torus with its edges numbered two ways: identical facets, first points and
    point sources from the shared-point bookkeeping."""
    cage = shapes.torus(10, 6, tri_fraction=0.2, seed=5)
    sizes, fv = cage.verts_per_face, cage.face_verts
    ro, rates = workloads.bfr_edge_length_rates(cage.positions, sizes, fv, 0.05, 6)
    mesh = oracle.tess_mesh(4, sizes, ro, rates)
    fe, ne = workloads.face_edges(sizes, fv)
    perm = np.random.default_rng(3).permutation(ne).astype(np.int32)
    a = oracle.tess_share(4, sizes, fv, fe, cage.num_vertices, ne, ro, rates,
                          mesh["coord_offsets"], mesh["facet_offsets"], mesh["facets"])
    b = oracle.tess_share(4, sizes, fv, perm[fe], cage.num_vertices, ne, ro, rates,
                          mesh["coord_offsets"], mesh["facet_offsets"], mesh["facets"])
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    # each point is made from its own coord, and every coord index of a facet became a point
    facets, po, src = a
    assert len(src) == len(np.unique(src))
    assert facets.min() >= 0 and facets.max() == len(src) - 1
