"""Drop-in for pyaxisymflow/elasto_kernels/div_tau.py:4-34."""
from .. import _native as N


def update_vorticity_from_solid_stress(vorticity, tau_z, tau_r, tau11, tau12, tau22, R, dt, dx):
    """vorticity[1:-1, 1:-1] += dt * curl(div tau), tau_z / tau_r are outputs."""
    s = N.require(vorticity, tau_z, tau_r, tau11, tau12, tau22, R, shape=vorticity.shape,
                  names=("vorticity", "tau_z", "tau_r", "tau11", "tau12", "tau22", "R"))
    nr, nz = vorticity.shape
    N.call(f"axi_update_vorticity_from_solid_stress_{s}", N.ptr(vorticity), N.ptr(tau_z),
           N.ptr(tau_r), N.ptr(tau11), N.ptr(tau12), N.ptr(tau22), N.ptr(R), nr, nz,
           N.real(s, dt), N.real(s, dx), N.stream_of(vorticity))
