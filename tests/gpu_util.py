"""Helpers shared by the GPU parity tests."""
import numpy as np


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return d / n if n > 0 else d


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
