"""The native uniform-refinement stencil generator (the benchmark's workload source) against
the reference's own Far::StencilTableFactory tables stored in the golden fixtures.

Rows are matched by the refined point they produce on random control data (the generator
orders child vertices like Vtr but its child-edge numbering may differ), then compared as
sparse rows: identical supports and weights within 2 float ulps of 1.
"""
import glob
import os

import numpy as np
import pytest
from scipy.spatial import cKDTree

from opensubdiv_gb300 import shapes, topology

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# the generator takes closed cages with creases only: the reference's regression shapes (open
# boundaries, corner tags, non-manifold edges; reg_*) are outside its domain
FIXTURES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*_uniform_L*.npz"))
                  if not os.path.basename(p).startswith("reg_"))


def _cage(z):
    return shapes.Cage(z["positions"], z["verts_per_face"], z["face_verts"], int(z["scheme"]),
                       z["crease_verts"], z["crease_sharpness"])


def _apply(t, X):
    n = len(t["sizes"])
    rows = np.repeat(np.arange(n), t["sizes"])
    Y = np.zeros((n, X.shape[1]))
    np.add.at(Y, rows, t["weights"][:, None].astype(np.float64) * X[t["indices"]])
    return Y


def _row(t, i):
    o, s = t["offsets"][i], t["sizes"][i]
    return dict(zip(t["indices"][o:o + s].tolist(), t["weights"][o:o + s].tolist()))


@pytest.mark.parametrize("path", FIXTURES, ids=os.path.basename)
def test_generator_reproduces_far_stencil_tables(path):
    z = np.load(path)
    cage = _cage(z)
    level = int(z["level"])
    mine = topology.UniformRefiner(cage, level).stencil_table()
    far = dict(sizes=z["sizes"], offsets=z["offsets"], indices=z["indices"], weights=z["weights"])
    assert len(mine["sizes"]) == len(far["sizes"])
    assert len(mine["indices"]) == len(far["indices"])
    X = np.random.default_rng(0).normal(size=(cage.num_vertices, 4))
    d, j = cKDTree(_apply(far, X)).query(_apply(mine, X))
    assert d.max() < 1e-5
    assert len(np.unique(j)) == len(j)  # a permutation
    for i in range(len(j)):
        a, b = _row(mine, i), _row(far, j[i])
        assert set(a) == set(b)
        assert max(abs(a[k] - b[k]) for k in a) <= 2.4e-7


def test_generator_limit_stencils_match_far_on_a_uniform_refiner():
    """The generator's limit stencils (config 2's limit pass) against the table
    Far::LimitStencilTableFactory builds on the same uniform refiner at the same locations
    (far/stencilTableFactory.cpp:411-662; tests/golden/uniform_limit_pin.npz): the same
    supports, with P / du / dv weights within float rounding."""
    z = np.load(os.path.join(GOLDEN, "uniform_limit_pin.npz"))
    cage = _cage(z)
    mine = topology.UniformRefiner(cage, int(z["level"])).limit_stencil_table(z["face"], z["u"],
                                                                            z["v"])
    assert np.array_equal(mine["sizes"], z["sizes"])
    for key in ("weights", "du_weights", "dv_weights"):
        a = dict(sizes=mine["sizes"], offsets=mine["offsets"], indices=mine["indices"],
                 weights=mine[key])
        b = dict(sizes=z["sizes"], offsets=z["offsets"], indices=z["indices"], weights=z[key])
        for i in range(len(z["sizes"])):
            ra, rb = _row(a, i), _row(b, i)
            assert set(ra) == set(rb), (key, i)
            assert max(abs(ra[k] - rb[k]) for k in ra) <= 2e-6 * max(1.0, max(map(abs, rb.values()))), (key, i)


def test_generator_limit_stencils_are_bilinear_partitions():
    """Limit stencils of a uniform refiner: position weights sum to 1, du/dv weights to 0."""
    cage = shapes.torus(16, 8, tri_fraction=0.1, crease_fraction=0.05, seed=3)
    r = topology.UniformRefiner(cage, 2)
    face, u, v = shapes.uniform_locations(cage, 500, seed=4)
    t = r.limit_stencil_table(face, u, v)
    assert len(t["sizes"]) == 500
    rows = np.repeat(np.arange(500), t["sizes"])
    for key, target in (("weights", 1.0), ("du_weights", 0.0), ("dv_weights", 0.0)):
        s = np.zeros(500)
        np.add.at(s, rows, t[key].astype(np.float64))
        assert np.abs(s - target).max() < 1e-5, key


def test_generator_rejects_open_cages():
    with pytest.raises(ValueError):
        topology.UniformRefiner(shapes.grid(3, 3), 1)


@pytest.mark.parametrize("scheme", ["catmark", "loop"])
def test_generator_far_form_masks_compose_to_its_tables(scheme):
    """The generator's masks in Far::PrimvarRefiner form (the GPU factory's input), merged as
    Far's StencilBuilder does (the oracle), give the generator's own tables: same stencils and
    supports, weights within 2 float ulps of 1 (float vs double accumulation)."""
    import oracle
    if scheme == "catmark":
        cage = shapes.torus(16, 8, tri_fraction=0.1, crease_fraction=0.05, seed=3)
    else:
        cage = shapes.torus(12, 8, crease_fraction=0.05, seed=4, scheme=shapes.LOOP)
    r = topology.UniformRefiner(cage, 3)
    mine = r.stencil_table()
    nc, levels = r.factory_masks()
    first = nc
    for d in levels:
        n = len(d["offsets"]) - 1
        assert d["sources"].min() >= 0 and d["sources"].max() < first + n
        assert (d["sources"] >= first).any() == (scheme == "catmark")  # face points
        first += n
    t = oracle.factory_create(nc, levels, intermediate=False)
    assert np.array_equal(t["sizes"], mine["sizes"])
    for i in range(len(t["sizes"])):
        a, b = _row(t, i), _row(mine, i)
        assert set(a) == set(b)
        assert max(abs(a[k] - b[k]) for k in a) <= 2.4e-7
