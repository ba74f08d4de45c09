"""The C++ drop-in header (include/opensubdiv_gb300/osd/gb300Evaluator.h) used by a compiled
C++ client on the GPU: table + vertex buffer + template EvalStencils, checked against the
oracle (= Osd::CpuEvaluator bit for bit)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle

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
    """Device PatchMap, EvalPatches (P, du, dv) and EvalPatchesFaceVarying from C++ through
    the header, on the reference's face-varying torus table."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    z = np.load(os.path.join(GOLDEN, "torus12x8_fvar_patches_L3.npz"))
    for k in ("arrays", "patch_indices", "params", "varying_arrays", "varying_indices",
              "fvar_arrays", "fvar_indices", "fvar_params", "src", "fvar_src", "q_face", "q_u",
              "q_v"):
        np.ascontiguousarray(z[k]).tofile(tmp_path / f"{k}.bin")
    np.array([int(z["triangular"])], np.int32).tofile(tmp_path / "triangular.bin")
    exe = _build(tmp_path, "dropin_patches")
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    nq = len(z["q_face"])
    handles = np.fromfile(tmp_path / "handles.bin", np.int32).reshape(nq, 3)
    assert np.array_equal(handles, z["q_handles"])
    hit = z["q_found"].astype(bool)
    A = oracle.abs_scale(z["src"], (0, 3, 3), 3, z["coords"], z["arrays"], z["patch_indices"],
                         z["params"])
    for k, name in enumerate(("p", "du", "dv")):
        out = np.fromfile(tmp_path / f"{name}.bin", np.float32).reshape(nq, 3)
        assert np.all(out[~hit] == 0)
        bound = 1e-6 * np.maximum(A[k].reshape(-1, 3), 1.0)
        assert np.all(np.abs(out[hit] - z["out6"][k]) <= bound), name
    fv = np.fromfile(tmp_path / "fvar.bin", np.float32).reshape(nq, 2)
    Af = oracle.abs_scale(z["fvar_src"], (0, 2, 2), 2, z["coords"], z["fvar_arrays"],
                          z["fvar_indices"], z["fvar_params"])
    assert np.all(np.abs(fv[hit] - z["fvar_out6"][0]) <= 1e-6 * np.maximum(Af[0].reshape(-1, 2), 1.0))
