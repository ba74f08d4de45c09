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
