"""Helpers shared by the GPU tests: device copies in the reference layout and
the float error measures."""
import hashlib

import numpy as np

import inputs

BOUND = {"float": 2e-7, "double": 1e-15}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def to_dev(a):
    import torch
    a = np.ascontiguousarray(a)
    if np.iscomplexobj(a):
        a = a.view(np.float32 if a.dtype == np.complex64 else np.float64)
    return torch.from_numpy(a.copy()).cuda()


def empty_dev(like_np):
    import torch
    a = like_np
    if np.iscomplexobj(a):
        a = a.view(np.float32 if a.dtype == np.complex64 else np.float64)
    return torch.zeros(a.shape, dtype=getattr(torch, a.dtype.name), device="cuda")


def from_dev(t, like_np):
    import torch
    torch.cuda.synchronize()
    a = t.cpu().numpy()
    if np.iscomplexobj(like_np):
        a = a.view(like_np.dtype)
    return a.reshape(like_np.shape)


def relerr_rows(got, exact):
    got = got.reshape(exact.shape[0], -1)
    exact = exact.reshape(exact.shape[0], -1)
    e = np.linalg.norm(got - exact, axis=1)
    s = np.linalg.norm(exact, axis=1)
    s[s == 0] = 1
    return float(np.max(e / s))


def bound(dtype, n):
    return BOUND[dtype] * max(1.0, float(np.log2(max(n, 2))))


def c128(a, dtype):
    return inputs.to_complex128(a, dtype)
