"""Helpers for the GPU tests: device copies through torch (allocation only; all compute is in
libagb_cuda) and tolerance reports."""
import numpy as np


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def empty(shape, dtype):
    import torch
    return torch.zeros(shape, dtype=dtype, device="cuda")


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def rel_err(a, b, floor):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)
