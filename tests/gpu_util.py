"""Shared helpers for the GPU parity tests (device memory via torch, checks via the oracle)."""
from __future__ import annotations

import numpy as np


def torch_cuda():
    import torch

    if not torch.cuda.is_available():
        import pytest

        pytest.skip("no CUDA device")
    return torch


def dev(a, torch=None):
    torch = torch or torch_cuda()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def bbox_diag(positions):
    p = np.asarray(positions, np.float64).reshape(-1, 3)
    return float(np.linalg.norm(p.max(0) - p.min(0)))


def max_err(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.abs(a - b).max()) if a.size else 0.0


# ---- the accuracy gate ---------------------------------------------------------------------
#
# Every float output is held to the bound 1e-5 x the bounding-box diagonal of the evaluated
# points ("flat", no scaling):
#   - P, dPdu, dPdv: max |gpu - cpu| <= flat, cpu = Osd::CpuEvaluator (the oracle reproduces it
#     bit for bit);
#   - dPduu, dPduv, dPdvv: max |gpu - fp64| <= flat, fp64 = the same tables and bases applied
#     in double.  The reference's own float evaluation is not within flat of FP64 for these
#     outputs (its cancelling sums carry the 4^depth factor), so no float evaluation can be
#     within flat of it in general; the GPU must instead be closer to the exact result than
#     the bound, and its distance from the CPU is then at most |cpu - fp64| + flat, which is
#     asserted too.
# Stencil tables carry their derivative weights as given floats, applied in the reference's
# order: there every output, second derivatives included, is held to |gpu - cpu| <= flat
# (gate(..., all_vs_cpu=True)), with the float table applied in double reported beside it.
# Each check appends (case, output, |gpu-cpu|, |gpu-fp64|, |cpu-fp64|, flat) to REPORT; a run
# with OSD_GB300_ERROR_REPORT=<path> writes them as JSON (tests/conftest.py).
REL_TOL = 1e-5
OUTPUT_NAMES = ("P", "du", "dv", "duu", "duv", "dvv")
REPORT = []


def bbox_diag_rows(src, length, desc=None):
    """Bounding-box diagonal of the rows of a primvar buffer (length elements per row)."""
    s = np.asarray(src, np.float64).ravel()
    if desc is not None:
        off, ln, st = desc
        rows = (len(s) - off) // st
        s = np.stack([s[off + k: off + k + rows * st: st] for k in range(ln)], 1)
    else:
        s = s.reshape(-1, length)
    return float(np.linalg.norm(s.max(0) - s.min(0)))


def gate(case, k, gpu, cpu, fp64, diag, all_vs_cpu=False):
    """Asserts the accuracy contract for output k (0..5) and records the errors."""
    flat = REL_TOL * diag
    e_cpu = max_err(gpu, cpu)
    e_f64 = max_err(gpu, fp64) if fp64 is not None else float("nan")
    c_f64 = max_err(cpu, fp64) if fp64 is not None else float("nan")
    REPORT.append(dict(case=case, output=OUTPUT_NAMES[k], gpu_cpu=e_cpu, gpu_fp64=e_f64,
                       cpu_fp64=c_f64, flat=flat))
    if k < 3 or all_vs_cpu:
        assert e_cpu <= flat, f"{case} {OUTPUT_NAMES[k]}: |gpu-cpu| {e_cpu:.3e} > {flat:.3e}"
    else:
        assert fp64 is not None, "second derivatives are gated against FP64"
        assert e_f64 <= flat, f"{case} {OUTPUT_NAMES[k]}: |gpu-fp64| {e_f64:.3e} > {flat:.3e}"
        assert e_cpu <= c_f64 + flat, f"{case} {OUTPUT_NAMES[k]}: |gpu-cpu| {e_cpu:.3e}"


def smooth_primvars(xyz, width=8, lane=2):
    """`width` interleaved primvars over points xyz [n, 3]: xyz in lanes lane..lane+2 and
    smooth O(1) functions of position in the others (colours, texture coordinates and
    normals vary smoothly over a surface)."""
    x, y, z = (np.asarray(xyz, np.float64)[:, i] for i in range(3))
    extra = [np.sin(2 * x) * np.cos(3 * y), x * y - z, np.cos(2 * z) + 0.5 * x, x * x - y * y,
             0.3 * (x + y + z), np.sin(y + z), x * z, np.cos(x - y)]
    out = np.zeros((len(x), width), np.float32)
    j = 0
    for c in range(width):
        if lane <= c < lane + 3:
            out[:, c] = xyz[:, c - lane]
        else:
            out[:, c] = extra[j % len(extra)]
            j += 1
    return out


def serving_bases():
    """The serving pool's base shapes from the fixtures (the reference's adaptive tables of the
    32 x 16 torus and the level-2 icosphere)."""
    import os

    from opensubdiv_gb300 import shapes, workloads
    g = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    return {shapes.CATMARK: workloads.ServingBase(np.load(os.path.join(g, "torus32x16_patches_L4.npz"))),
            shapes.LOOP: workloads.ServingBase(np.load(os.path.join(g, "icosphere2_patches_L3.npz")))}
