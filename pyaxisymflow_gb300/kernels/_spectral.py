"""Shared engine of the fast-diagonalisation solvers.

Setup runs once on the host in FP64, as in the reference: the 1-D finite
difference operators are built, edited for the boundary conditions and
eigendecomposed with LAPACK (numpy.linalg.eig, descending eigenvalue order,
kernels/FastDiagonalisationStokesSolver.py:99-128). The eigenbases are
uploaded once and every solve runs on the GPU as four dense products
(include/axisym_gb300.h: axi_fd_transform_f64).

numpy >= 2 returns complex eigenvectors even when all imaginary parts are
zero (the numpy the reference pins returned real ones then); the imaginary
parts are checked to be exactly zero and dropped.
"""
import numpy as np
import torch

from .. import _native as N


def tridiag(n, lo, d, up):
    m = np.zeros((n, n))
    i = np.arange(n)
    m[i, i] = d
    m[i[1:], i[:-1]] = lo
    m[i[:-1], i[1:]] = up
    return m


def eig_sorted_desc(mat):
    vals, vecs = np.linalg.eig(mat)
    idx = vals.argsort()[::-1]
    vals, vecs = vals[idx], vecs[:, idx]
    for a in (vals, vecs):
        if np.iscomplexobj(a) and np.any(a.imag != 0):
            raise ValueError("eigendecomposition has a non-zero imaginary part")
    return np.ascontiguousarray(np.real(vals)), np.ascontiguousarray(np.real(vecs))


def radial_coord(dx, nr):
    return np.linspace(dx / 2, nr * dx - dx / 2, nr).reshape(nr, 1)


def _row_stride(t, nr, nz, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (there is no CPU path)")
    if tuple(t.shape) != (nr, nz):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {(nr, nz)}")
    if t.dtype != torch.float64:
        raise TypeError(f"{name} must be float64 (got {t.dtype})")
    if t.stride(1) != 1 or t.stride(0) < nz:
        raise ValueError(f"{name} must have unit z stride and row stride >= nz")
    return t.stride(0)


class FastDiagonalisationEngine:
    """Device copy of one eigenbasis set and the transform that applies it."""

    def __init__(self, eig_vals_r, eig_vecs_r, eig_vals_z, eig_vecs_z, spectrum, row_weight,
                 device=None):
        nr, nz = spectrum.shape
        self.grid_size_r, self.grid_size_z = nr, nz
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None \
            else torch.device(device)
        self.device = dev
        inv_r = np.linalg.inv(eig_vecs_r)
        if row_weight is not None:
            inv_r = inv_r * row_weight.reshape(1, nr)
        host = dict(
            Er=eig_vecs_r,
            Er_inv_w=inv_r,
            EzinvT=np.linalg.inv(eig_vecs_z).T,
            EzT=eig_vecs_z.T,
            inv_eig=1.0 / spectrum,
        )
        self.host = host
        self.eig_vals_r, self.eig_vals_z = eig_vals_r, eig_vals_z
        self.dev = {k: torch.tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev)
                    for k, v in host.items()}
        self.work = torch.empty(2 * nr * nz, dtype=torch.float64, device=dev)

    def transform(self, out, inp):
        nr, nz = self.grid_size_r, self.grid_size_z
        ld_in = _row_stride(inp, nr, nz, "rhs_field")
        ld_out = _row_stride(out, nr, nz, "solution_field")
        d = self.dev
        N.call("axi_fd_transform_f64", N.ptr(out), ld_out, N.ptr(inp), ld_in,
               N.ptr(d["Er_inv_w"]), N.ptr(d["EzinvT"]), N.ptr(d["inv_eig"]), N.ptr(d["Er"]),
               N.ptr(d["EzT"]), N.ptr(self.work), nr, nz, N.stream_of(out))
