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
import ctypes

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


def tf32_round(x32):
    """Nearest TF32 value (10 explicit mantissa bits, ties away from zero) of a
    float32 array, as float32."""
    b = np.ascontiguousarray(x32, dtype=np.float32).view(np.uint32)
    return ((b + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)


def tf32_split(x):
    """Operand pair of the 3xTF32 products from a float64 array: hi = nearest
    TF32 of fl32(x), lo = nearest TF32 of fl32(x - hi) (remainder in double);
    hi + lo carries about 23 significant bits."""
    x64 = np.asarray(x, dtype=np.float64)
    hi = tf32_round(x64.astype(np.float32))
    lo = tf32_round((x64 - hi.astype(np.float64)).astype(np.float32))
    return hi, lo


def tridiagonals(mat):
    """(sub, main, super) diagonal of each row of a tridiagonal matrix."""
    n = mat.shape[0]
    out = np.zeros((n, 3))
    i = np.arange(n)
    out[:, 1] = mat[i, i]
    out[1:, 0] = mat[i[1:], i[1:] - 1]
    out[:-1, 2] = mat[i[:-1], i[:-1] + 1]
    return out


class AxiTcTransform(ctypes.Structure):
    """Mirror of ``axi_tc_transform`` in include/axisym_gb300.h."""
    _fields_ = [("nr", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("basis", ctypes.c_void_p * 8), ("inv_eig", ctypes.c_void_p),
                ("in_hi", ctypes.c_void_p), ("in_lo", ctypes.c_void_p),
                ("work", ctypes.c_void_p * 4), ("out", ctypes.c_void_p)]


class AxiTcPlanInfo(ctypes.Structure):
    """Mirror of ``axi_tc_plan_info`` in include/axisym_gb300.h."""
    _fields_ = [("n", ctypes.c_int32), ("n_tiles", ctypes.c_int32 * 4),
                ("reserved", ctypes.c_int32), ("bytes", ctypes.c_int64)]


class FastDiagonalisationEngine:
    """Device copy of one eigenbasis set and the transform that applies it.

    precision "f64": four FP64 products (axi_fd_transform_f64).
    precision "f32": four tcgen05 3xTF32 products (axi_tc_transform_run), then
    `refine` steps of iterative refinement with the residual of the discrete
    operator A_r (x) I + I (x) A_z computed in FP64 (op_r, op_z are those
    1-D matrices, wrap entries included).
    """

    def __init__(self, eig_vals_r, eig_vecs_r, eig_vals_z, eig_vecs_z, spectrum, row_weight,
                 device=None, precision="f64", op_r=None, op_z=None, refine=1):
        nr, nz = spectrum.shape
        self.grid_size_r, self.grid_size_z = nr, nz
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None \
            else torch.device(device)
        self.device = dev
        self.precision = precision
        self.refine = refine
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
        if precision == "f64":
            self.dev = {k: torch.tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev)
                        for k, v in host.items()}
            self.work = torch.empty(2 * nr * nz, dtype=torch.float64, device=dev)
        elif precision == "f32":
            self._setup_tc(host, row_weight, op_r, op_z)
        else:
            raise ValueError("precision must be 'f64' or 'f32'")

    def _setup_tc(self, host, row_weight, op_r, op_z):
        nr, nz = self.grid_size_r, self.grid_size_z
        if nr % 4 or nz % 4:
            raise ValueError("the tensor-core solve needs nr and nz multiples of 4")
        dev = self.device
        f32 = dict(dtype=torch.float32, device=dev)
        f64 = dict(dtype=torch.float64, device=dev)
        self.tc_basis = []
        for m in (host["EzinvT"].T, host["Er_inv_w"], host["EzT"].T, host["Er"]):
            hi, lo = tf32_split(np.ascontiguousarray(m))
            self.tc_basis += [torch.tensor(hi, device=dev), torch.tensor(lo, device=dev)]
        self.tc_inv_eig = torch.tensor(host["inv_eig"], **f32)
        self.tc_in = [torch.empty((nr, nz), **f32) for _ in range(2)]
        self.tc_work = [torch.empty(nr * nz, **f32) for _ in range(4)]
        self.tc_out = torch.empty((nr, nz), **f32)
        self.tc_psi = torch.empty((nr, nz), **f64)
        self.tc_res = torch.empty((nr, nz), **f64)
        self.weight = (torch.tensor(np.ascontiguousarray(row_weight), **f64)
                       if row_weight is not None else None)
        self.op_r = torch.tensor(tridiagonals(op_r), **f64) if op_r is not None else None
        self.op_z = torch.tensor(tridiagonals(op_z), **f64) if op_z is not None else None
        self.wrap = (float(op_z[0, -1]), float(op_z[-1, 0])) if op_z is not None else (0.0, 0.0)
        t = AxiTcTransform()
        t.nr, t.nz = nr, nz
        for q in range(8):
            t.basis[q] = self.tc_basis[q].data_ptr()
        t.inv_eig = self.tc_inv_eig.data_ptr()
        t.in_hi, t.in_lo = self.tc_in[0].data_ptr(), self.tc_in[1].data_ptr()
        for q in range(4):
            t.work[q] = self.tc_work[q].data_ptr()
        t.out = self.tc_out.data_ptr()
        self.tc_t = t
        self.tc_info = AxiTcPlanInfo()
        s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        N.call("axi_tc_transform_plan", ctypes.byref(t), 1, None, ctypes.byref(self.tc_info), s)
        self.tc_plan = torch.empty(int(self.tc_info.bytes), dtype=torch.uint8, device=dev)
        N.call("axi_tc_transform_plan", ctypes.byref(t), 1, N.ptr(self.tc_plan),
               ctypes.byref(self.tc_info), s)

    def _tc_run(self, s):
        N.call("axi_tc_transform_run", ctypes.byref(self.tc_info), N.ptr(self.tc_plan), s)

    def tc_status(self):
        err = ctypes.c_int(0)
        N.call("axi_tc_transform_status", ctypes.byref(self.tc_info), N.ptr(self.tc_plan),
               ctypes.byref(err), ctypes.c_void_p(torch.cuda.current_stream(
                   self.device).cuda_stream))
        return err.value

    def transform(self, out, inp):
        nr, nz = self.grid_size_r, self.grid_size_z
        if self.precision == "f32":
            self._transform_tc(out, inp)
            return
        ld_in = _row_stride(inp, nr, nz, "rhs_field")
        ld_out = _row_stride(out, nr, nz, "solution_field")
        d = self.dev
        N.call("axi_fd_transform_f64", N.ptr(out), ld_out, N.ptr(inp), ld_in,
               N.ptr(d["Er_inv_w"]), N.ptr(d["EzinvT"]), N.ptr(d["inv_eig"]), N.ptr(d["Er"]),
               N.ptr(d["EzT"]), N.ptr(self.work), nr, nz, N.stream_of(out))

    def _transform_tc(self, out, inp):
        nr, nz = self.grid_size_r, self.grid_size_z
        for t, name in ((inp, "rhs_field"), (out, "solution_field")):
            if not isinstance(t, torch.Tensor) or not t.is_cuda:
                raise ValueError(f"{name} must be a CUDA tensor (there is no CPU path)")
            if tuple(t.shape) != (nr, nz) or t.dtype not in (torch.float32, torch.float64):
                raise ValueError(f"{name} must be a float32 / float64 tensor of shape {(nr, nz)}")
        s = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        x = inp.contiguous()
        n = nr * nz
        hi, lo = self.tc_in
        if x.dtype == torch.float64:
            N.call("axi_tc_split_f64", N.ptr(hi), N.ptr(lo), N.ptr(x), n, s)
        else:
            N.call("axi_tc_split_f32", N.ptr(hi), N.ptr(lo), N.ptr(x), n, s)
        self._tc_run(s)
        if not self.refine:
            out.copy_(self.tc_out)
            return
        if self.op_r is None:
            raise ValueError("refinement needs the discrete operator")
        psi, res = self.tc_psi, self.tc_res
        N.call("axi_widen_f32_to_f64", N.ptr(psi), N.ptr(self.tc_out), n, s)
        x64 = x if x.dtype == torch.float64 else x.double()
        for _ in range(self.refine):
            N.call("axi_fd_residual_f64", N.ptr(res), N.ptr(x64), N.ptr(psi),
                   N.ptr(self.weight) if self.weight is not None else None, N.ptr(self.op_r),
                   N.ptr(self.op_z), nr, nz, self.wrap[0], self.wrap[1], s)
            N.call("axi_tc_split_f64", N.ptr(hi), N.ptr(lo), N.ptr(res), n, s)
            self._tc_run(s)
            N.call("axi_add_f32_to_f64", N.ptr(psi), N.ptr(self.tc_out), n, s)
        out.copy_(psi)
