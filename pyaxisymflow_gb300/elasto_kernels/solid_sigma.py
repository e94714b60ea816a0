"""Drop-in for pyaxisymflow/elasto_kernels/solid_sigma.py:4-29."""
from .. import _native as N


def solid_sigma(sigma_s_11, sigma_s_12, sigma_s_22, G, dx, eta_1, eta_2, eta_1z, eta_1r,
                eta_2z, eta_2r):
    """neo-Hookean solid stress from reference-map gradients (gradient arrays
    are written where the reference writes them)."""
    s = N.require(sigma_s_11, sigma_s_12, sigma_s_22, eta_1, eta_2, eta_1z, eta_1r, eta_2z,
                  eta_2r, shape=eta_1.shape,
                  names=("sigma_s_11", "sigma_s_12", "sigma_s_22", "eta_1", "eta_2", "eta_1z",
                         "eta_1r", "eta_2z", "eta_2r"))
    nr, nz = eta_1.shape
    N.call(f"axi_solid_sigma_{s}", N.ptr(sigma_s_11), N.ptr(sigma_s_12), N.ptr(sigma_s_22),
           N.real(s, G), N.real(s, dx), N.ptr(eta_1), N.ptr(eta_2), N.ptr(eta_1z), N.ptr(eta_1r),
           N.ptr(eta_2z), N.ptr(eta_2r), nr, nz, N.stream_of(eta_1))
