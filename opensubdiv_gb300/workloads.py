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


def refine_cube(n=8, level=4, seed=1):
    cage = shapes.cube(n, noise=0.01, seed=seed)
    refine = UniformRefiner(cage, level).stencil_table()
    return dict(name=f"cube{n}_catmark_L{level}_xyz", cage=cage,
                src=np.ascontiguousarray(cage.positions.ravel()), length=3, refine=refine,
                level=level)
