"""Batched Newton iteration-matrix algebra on the GPU (the scipy dgetrf/dgetrs pair of the reference's
HomogeneousReactor linear setup/solve, reactors.py:340-356, for a whole batch of states).

``NewtonSystems`` factors A_k = gamma_h[k] J_k - I for n states (FP64 LU, or FP32 LU of the FP64 matrix) and
solves A_k x_k = b_k (FP32 triangular solves followed by FP64 residual-refinement sweeps in the FP32 variant).
"""

import numpy as np

from . import _native as N


def _torch():
    import torch
    return torch


class NewtonSystems:
    def __init__(self, n, m, precision=0, refine=2, device=None):
        torch = _torch()
        if precision not in (0, 1):
            raise ValueError('precision must be 0 (FP64 LU) or 1 (FP32 LU + FP64 refinement)')
        dev = device or torch.device('cuda', torch.cuda.current_device())
        self.n, self.m, self.precision, self.refine = n, m, precision, refine
        self.A = torch.empty((n, m * m), dtype=torch.float64, device=dev)
        self.lu = torch.empty((n, m * m), dtype=torch.float64 if precision == 0 else torch.float32, device=dev)
        self.piv = torch.empty((n, m), dtype=torch.int32, device=dev)
        self.info = torch.empty(n, dtype=torch.int32, device=dev)

    def factor(self, J, gamma_h):
        """J: [n, m*m] column-major Jacobians (CUDA FP64); gamma_h: [n] CUDA FP64."""
        N.check(N.load().sf_newton_lu_batch(self.n, self.m, N.ptr(J), N.ptr(gamma_h), self.precision,
                                            N.ptr(self.A), N.ptr(self.lu), N.ptr(self.piv), N.ptr(self.info),
                                            N.stream_handle()))
        return self

    def solve(self, b, out=None, start=0, count=None):
        """Solve systems start .. start+count-1 (all by default) for the rows of b ([count, m])."""
        import ctypes as C
        torch = _torch()
        count = self.n - start if count is None else count
        if not (0 <= start and count >= 0 and start + count <= self.n) or b.shape[0] != count:
            raise ValueError('system range out of bounds or right-hand sides of the wrong count')
        out = torch.empty_like(b) if out is None else out
        mm = self.m * self.m
        esz = self.lu.element_size()
        N.check(N.load().sf_newton_solve_batch(count, self.m, C.c_void_p(self.A.data_ptr() + start * mm * 8),
                                               C.c_void_p(self.lu.data_ptr() + start * mm * esz),
                                               C.c_void_p(self.piv.data_ptr() + start * self.m * 4),
                                               self.precision, self.refine, N.ptr(b), N.ptr(out),
                                               N.stream_handle()))
        return out


def backward_error(A, x, b):
    """Normwise backward error |b - A x|_inf / (|A|_inf |x|_inf + |b|_inf) per system (host numpy arrays;
    A: [n, m, m] row-major)."""
    res = np.abs(b - np.einsum('kij,kj->ki', A, x)).max(1)
    return res / (np.abs(A).sum(2).max(1) * np.abs(x).max(1) + np.abs(b).max(1))
