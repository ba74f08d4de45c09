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
