"""The C++ drop-in header (include/opensubdiv_gb300/osd/gb300Evaluator.h) used by a compiled
C++ client on the GPU: table + vertex buffer + template EvalStencils, checked against the
oracle (= Osd::CpuEvaluator bit for bit)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from gpu_util import bbox_diag, bbox_diag_rows, gate

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def test_header_compiles_standalone(tmp_path):
    """Without OpenSubdiv on the include path the header declares layout-identical Osd
    types and still compiles (CPU-only check)."""
    src = os.path.join(ROOT, "tests", "cpp", "dropin_client.cpp")
    cuda = _cuda_home()
    r = subprocess.run(["g++", "-std=c++14", "-fsyntax-only", f"-I{ROOT}/include",
                        f"-I{cuda}/include", src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cpp_client_through_drop_in_header(tmp_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from opensubdiv_gb300 import _lib
    _lib.load()
    z = np.load(os.path.join(GOLDEN, "cube8_uniform_L3.npz"))
    for k in ("sizes", "offsets", "indices", "weights"):
        z[k].tofile(tmp_path / f"{k}.bin")
    z["positions"].astype(np.float32).tofile(tmp_path / "src.bin")
    exe = tmp_path / "dropin_client"
    cuda = _cuda_home()
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++14", "-O2", f"-I{ROOT}/include", f"-I{cuda}/include",
                        os.path.join(ROOT, "tests", "cpp", "dropin_client.cpp"), "-o", str(exe),
                        f"-L{libdir}", "-losd_gb300", f"-Wl,-rpath,{libdir}", f"-L{cuda}/lib64",
                        "-lcudart", f"-Wl,-rpath,{cuda}/lib64"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.fromfile(tmp_path / "out.bin", np.float32)
    n = len(z["sizes"])
    ref = np.zeros(n * 3, np.float32)
    oracle.eval_stencils(z["positions"].ravel(), (0, 3, 3), [ref], [(0, 3, 3)], z["sizes"],
                         z["offsets"], z["indices"], [z["weights"]])
    p = z["positions"].astype(np.float64)
    diag = float(np.linalg.norm(p.max(0) - p.min(0)))
    assert np.abs(out - ref).max() <= 1e-5 * diag


def _build(tmp_path, name):
    from opensubdiv_gb300 import _lib
    _lib.load()
    exe = tmp_path / name
    cuda = _cuda_home()
    libdir = os.path.dirname(_lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++14", "-O2", f"-I{ROOT}/include", f"-I{cuda}/include",
                        os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-o", str(exe),
                        f"-L{libdir}", "-losd_gb300", f"-Wl,-rpath,{libdir}", f"-L{cuda}/lib64",
                        "-lcudart", f"-Wl,-rpath,{cuda}/lib64"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_patch_client_header_compiles_standalone():
    src = os.path.join(ROOT, "tests", "cpp", "dropin_patches.cpp")
    cuda = _cuda_home()
    r = subprocess.run(["g++", "-std=c++14", "-fsyntax-only", f"-I{ROOT}/include",
                        f"-I{cuda}/include", src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cpp_patch_client_through_drop_in_header(tmp_path):
    """Device PatchMap, EvalPatches (P and all five derivatives), EvalPatchesVarying and
    EvalPatchesFaceVarying (all five derivatives) from C++ through the header's template forms,
    on the reference's face-varying torus table, and the same EvalPatches over a device table
    of the client's own type (the PATCH_TABLE type parameter)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    z = np.load(os.path.join(GOLDEN, "torus12x8_fvar_patches_L3.npz"))
    for k in ("arrays", "patch_indices", "params", "varying_arrays", "varying_indices",
              "fvar_arrays", "fvar_indices", "fvar_params", "src", "fvar_src", "varying_src",
              "q_face", "q_u", "q_v"):
        np.ascontiguousarray(z[k]).tofile(tmp_path / f"{k}.bin")
    np.array([int(z["triangular"])], np.int32).tofile(tmp_path / "triangular.bin")
    exe = _build(tmp_path, "dropin_patches")
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    nq = len(z["q_face"])
    handles = np.fromfile(tmp_path / "handles.bin", np.int32).reshape(nq, 3)
    assert np.array_equal(handles, z["q_handles"])
    hit = z["q_found"].astype(bool)
    diag = bbox_diag(z["positions"])
    for k in range(6):
        for tag in ("p", "g"):
            out = np.fromfile(tmp_path / f"{tag}{k}.bin", np.float32).reshape(nq, 3)
            assert np.all(out[~hit] == 0)
            gate(f"C++ client {'table' if tag == 'p' else 'client table'}", k, out[hit],
                 z["out6"][k], z["out6_fp64"][k], diag)
    dv_ = bbox_diag_rows(z["varying_src"], 4)
    for k in range(3):
        out = np.fromfile(tmp_path / f"var{k}.bin", np.float32).reshape(nq, 4)
        gate("C++ client varying", k, out[hit], z["varying_out3"][k], None, dv_)
    m = int(hit.sum())
    f64 = [np.zeros(m * 2) for _ in range(6)]
    oracle.eval_patches(z["fvar_src"], (0, 2, 2), f64, [(0, 2, 2)] * 6, z["coords"],
                        z["fvar_arrays"], z["fvar_indices"], z["fvar_params"], fp64=True)
    df = bbox_diag_rows(z["fvar_src"], 2)
    for k in range(6):
        fv = np.fromfile(tmp_path / f"fvar{k}.bin", np.float32).reshape(nq, 2)
        gate("C++ client face-varying", k, fv[hit], z["fvar_out6"][k], f64[k], df)


@pytest.mark.gpu
def test_cpp_client_second_derivative_stencils(tmp_path):
    """Limit stencils with all five derivatives from C++ through the header's six-output
    EvalStencils template: over a GB300StencilTable made from a Far::LimitStencilTable
    stand-in, and over a device table of the client's own type (the STENCIL_TABLE type
    parameter); the three-output form and a rejected descriptor as well."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    z = np.load(os.path.join(GOLDEN, "cube8_uniform_L3.npz"))
    names = ("weights", "du_weights", "dv_weights", "duu_weights", "duv_weights", "dvv_weights")
    for k in ("sizes", "offsets", "indices") + names:
        np.ascontiguousarray(z["limit_" + k]).tofile(tmp_path / f"limit_{k}.bin")
    z["positions"].astype(np.float32).tofile(tmp_path / "src.bin")
    exe = _build(tmp_path, "dropin_derivatives")
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    diag = bbox_diag(z["positions"])
    m = len(z["limit_sizes"])
    for k in range(6):
        f64 = np.zeros(m * 3)
        oracle.eval_stencils(z["positions"].ravel(), (0, 3, 3), [f64], [(0, 3, 3)],
                             z["limit_sizes"], z["limit_offsets"], z["limit_indices"],
                             [z["limit_" + names[k]]], fp64=True)
        for tag in ("a", "b"):
            out = np.fromfile(tmp_path / f"{tag}{k}.bin", np.float32)
            gate(f"C++ client limit stencils ({tag})", k, out, z["limit_out6"][k], f64, diag,
                 all_vs_cpu=True)
    c0 = np.fromfile(tmp_path / "c0.bin", np.float32)
    gate("C++ client limit stencils, 3 outputs", 0, c0, z["limit_out6"][0], None, diag)


def test_client_compiles_against_the_reference_far_headers(tmp_path):
    """A client written for CudaEvaluator -- Far::StencilTable, Far::LimitStencilTable with
    second derivatives and Far::PatchTable through the Osd template forms -- compiles against
    OpenSubdiv's own headers with only the type names changed (CPU-only check; needs the
    reference's source tree)."""
    refroot = os.environ.get("OPENSUBDIV_SOURCE", "/root/reference")
    if not os.path.isdir(os.path.join(refroot, "opensubdiv", "far")):
        pytest.skip("OpenSubdiv's headers are not available here")
    src = os.path.join(ROOT, "tests", "cpp", "dropin_far.cpp")
    obj = tmp_path / "dropin_far.o"
    cuda = _cuda_home()
    r = subprocess.run(["g++", "-std=c++14", "-O1", "-c", f"-I{refroot}", f"-I{ROOT}/include",
                        f"-I{cuda}/include", src, "-o", str(obj)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # and links against the reference's CPU library (Far, Osd::CpuPatchTable) and this one
    refdir = os.path.join(ROOT, "oracle", "_ref")
    from opensubdiv_gb300 import _lib
    if os.path.exists(os.path.join(refdir, "libosdref.so")) and os.path.exists(_lib.LIB_PATH):
        r = subprocess.run(["g++", "-o", str(tmp_path / "dropin_far"), str(obj), f"-L{refdir}",
                            "-losdref", f"-L{os.path.dirname(_lib.LIB_PATH)}", "-losd_gb300",
                            f"-L{cuda}/lib64", "-lcudart", "-fopenmp"],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_bfr_client_header_compiles_standalone():
    src = os.path.join(ROOT, "tests", "cpp", "bfr_client.cpp")
    cuda = _cuda_home()
    r = subprocess.run(["g++", "-std=c++14", "-fsyntax-only", f"-I{ROOT}/include",
                        f"-I{cuda}/include", src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["bfr_catmark_nonquads_e_f4q.npz", "bfr_torus16x8_e_f3.npz",
                                  "bfr_loop_xord_boundary_u5_f3.npz"])
def test_cpp_bfr_client_tessellates_like_bfr(tmp_path, name):
    """The Bfr tutorials' tessellate-and-evaluate loop from C++ through
    include/opensubdiv_gb300/bfr/gb300Tessellation.h and the evaluator header: coords and facets
    equal the reference's Bfr::Tessellation, PatchCoords its Far::PatchMap, and P..Dvv are within
    the reference's Bfr-versus-Far tolerances of Bfr::Surface::Evaluate."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    z = np.load(os.path.join(GOLDEN, name))
    for k in ("verts_per_face", "rate_offsets", "rates", "arrays", "patch_indices", "params",
              "src"):
        np.ascontiguousarray(z[k]).tofile(tmp_path / f"{k}.bin")
    np.array([int(z["regular_face_size"]), int(z["facet_size"]), int(z["preserve_quads"]),
              int(z["triangular"])], np.int32).tofile(tmp_path / "options.bin")
    import oracle
    fe, ne = oracle.edge_numbering(z["verts_per_face"], z["face_verts"])
    np.ascontiguousarray(z["face_verts"], np.int32).tofile(tmp_path / "face_verts.bin")
    np.ascontiguousarray(fe, np.int32).tofile(tmp_path / "face_edges.bin")
    np.array([len(z["positions"]), ne], np.int32).tofile(tmp_path / "topology.bin")
    exe = _build(tmp_path, "bfr_client")
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    n = len(z["coords"])
    coords = np.fromfile(tmp_path / "coords.bin", np.float32).reshape(n, 2)
    assert np.array_equal(coords.view(np.int32), z["coords"].view(np.int32))
    facets = np.fromfile(tmp_path / "facets.bin", np.int32).reshape(z["facets"].shape)
    assert np.array_equal(facets, z["facets"])
    pc = np.fromfile(tmp_path / "patch_coords.bin", np.int32).reshape(n, 5)
    assert np.array_equal(pc[:, :3], z["q_handles"])
    p = z["positions"].astype(np.float64)
    ptol = 5e-5 * float((p.max(0) - p.min(0)).max())
    for k, tol in enumerate((ptol, 5 * ptol, 5 * ptol, 25 * ptol, 25 * ptol, 25 * ptol)):
        out = np.fromfile(tmp_path / f"p{k}.bin", np.float32).reshape(n, 3)
        assert np.abs(out.astype(np.float64) - z["out6"][k]).max() <= tol, k
        if k < 3:  # the general EvalPatches entry on the same coords
            g = np.fromfile(tmp_path / f"g{k}.bin", np.float32).reshape(n, 3)
            assert np.abs(g.astype(np.float64) - z["out6"][k]).max() <= tol, k
    # shared points: the reference's tutorial 2.2 facets and numbering, P once per point
    share = np.load(os.path.join(GOLDEN, "bfr_share.npz"))
    key = name[:-4]
    sf = np.fromfile(tmp_path / "shared_facets.bin", np.int32).reshape(z["facets"].shape)
    assert np.array_equal(sf, share[key + "__facets"])
    po = np.fromfile(tmp_path / "point_offsets.bin", np.int64)
    assert np.array_equal(po, share[key + "__point_offsets"])
    src = share[key + "__point_sources"]
    pp = np.fromfile(tmp_path / "point_p.bin", np.float32).reshape(len(src), 3)
    p0 = np.fromfile(tmp_path / "p0.bin", np.float32).reshape(n, 3)
    assert np.array_equal(pp.view(np.int32), p0[src].view(np.int32))
