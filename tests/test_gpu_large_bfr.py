"""Bfr tessellate-and-evaluate at the benchmark's size: every face of the 512 x 256 torus
(137,628 faces, 5% triangles) at the Bfr tutorials' uniform rate 5, on the Far table of
Bfr::SurfaceFactory's default approximation (tests/golden/large/torus512x256_bfr.npz, written
where the reference is available by tests/golden/make_golden.py large).

All 4.8 M coords and 9.6 M facets must equal the oracle's (pinned to Bfr::Tessellation) bit for
bit; on the seeded 2% of faces the reference's Bfr evaluated, coords and facets equal
Bfr::Tessellation's and P, Du, Dv are within the reference's Bfr-versus-Far tolerances of
Bfr::Surface::Evaluate; and the located PatchCoords of every coord equal the oracle PatchMap's.
"""
import os

import numpy as np
import pytest

import oracle
from gpu_util import dev, host, torch_cuda

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "large",
                    "torus512x256_bfr.npz")


@pytest.mark.gpu
def test_full_mesh_rate5_against_oracle_and_bfr_sample():
    if not os.path.exists(PATH):
        pytest.skip("torus512x256_bfr.npz is written where the reference is available")
    torch_cuda()
    from opensubdiv_gb300 import bfr
    from opensubdiv_gb300.evaluator import BufferDescriptor as BD, GB300PatchTable
    z = np.load(PATH)
    sizes = z["verts_per_face"]
    nf = len(sizes)
    rate = int(z["rate"])
    table = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"], False)
    m = bfr.MeshTessellation(4, sizes, uniform_rate=rate)
    c, f, pc = m.Generate(table=table)
    c, f, pc = host(c), host(f), host(pc)
    t = oracle.tess_mesh(4, sizes, np.arange(nf + 1), np.full(nf, rate), 3, False, threads=16)
    assert np.array_equal(host(m.coord_offsets), t["coord_offsets"])
    assert np.array_equal(c.view(np.int32), t["coords"].view(np.int32))
    assert np.array_equal(f, t["facets"])
    ptex = host(m.ptex_offsets)
    qf, st = oracle.tess_locate_mesh(4, sizes, t["coord_offsets"], ptex, t["coords"], threads=16)
    pm = oracle.PatchMap(z["arrays"], z["params"], False)
    h = pm.find(qf, st[:, 0].astype(np.float64), st[:, 1].astype(np.float64))
    assert np.array_equal(pc[:, :3], h)
    assert np.array_equal(pc[:, 3], st[:, 0].view(np.int32))
    assert np.array_equal(pc[:, 4], st[:, 1].view(np.int32))

    # the reference's Bfr on its sample of faces
    outs = [host(o) for o in m.Evaluate(dev(z["src"]), BD(0, 3, 3), table, dev(pc), 1)]
    sel = np.nonzero(z["sample_rates"])[0]
    co = t["coord_offsets"]
    idx = np.concatenate([np.arange(co[i], co[i + 1]) for i in sel])
    assert np.array_equal(c[idx].view(np.int32), z["sample_coords"].view(np.int32))
    p = z["positions"].astype(np.float64)
    ptol = 5e-5 * float((p.max(0) - p.min(0)).max())
    for k, tol in enumerate((ptol, 5 * ptol, 5 * ptol)):
        err = np.abs(outs[k][idx].astype(np.float64) - z["sample_out3"][k]).max()
        assert err <= tol, (k, err, tol)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["uniform5", "edge_lengths"])
def test_full_mesh_shared_points_against_oracle(mode):
    """Shared (watertight) points of every face of the torus, at the uniform rate and at
    edge-length rates: facets, first points and point sources equal the oracle's bookkeeping
    (pinned to the reference's tutorial 2.2 loop by tests/test_bfr_oracle.py) exactly."""
    if not os.path.exists(PATH):
        pytest.skip("torus512x256_bfr.npz is written where the reference is available")
    torch_cuda()
    from opensubdiv_gb300 import bfr, workloads
    from opensubdiv_gb300.evaluator import GB300PatchTable
    z = np.load(PATH)
    sizes, fv = z["verts_per_face"], z["face_verts"]
    nf = len(sizes)
    table = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"], False)
    if mode == "uniform5":
        ro, rates = np.arange(nf + 1, dtype=np.int32), np.full(nf, int(z["rate"]), np.int32)
    else:
        ro, rates = workloads.bfr_edge_length_rates(z["positions"], sizes, fv, 0.0022)
    m = bfr.MeshTessellation(4, sizes, rates=rates, rate_offsets=ro)
    c, f, pc = m.Generate(table=table)
    t = oracle.tess_mesh(4, sizes, ro, rates, 3, False, threads=16)
    fe, ne = oracle.edge_numbering(sizes, fv)
    sp = m.Share(fv, fe, len(z["positions"]), ne, f, patch_coords=pc)
    want, po, src = oracle.tess_share(4, sizes, fv, fe, len(z["positions"]), ne, ro, rates,
                                      t["coord_offsets"], t["facet_offsets"], t["facets"])
    assert sp.num_points == len(src)
    assert np.array_equal(host(f), want)
    assert np.array_equal(host(sp.point_offsets), po)
    assert np.array_equal(host(sp.patch_coords), host(pc)[src])
