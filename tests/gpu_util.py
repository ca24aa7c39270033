import numpy as np


def to_dev(x):
    """numpy Fortran-order float64 -> column-major CUDA tensor (same values)."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).cuda().t()


def to_host(t):
    return np.asfortranarray(t.t().contiguous().cpu().numpy().T)


def load_alg(fmm, COEFFS, name):
    return fmm.new_fmm(COEFFS / f"{name}.txt")
