"""Drop-in for pyaxisymflow/kernels/implicit_diffusion_solver.py:6-143."""
import numpy as np

from ._spectral import FastDiagonalisationEngine, eig_sorted_desc, radial_coord, tridiag


class ImplicitEulerDiffusionStepper:
    """Implicit Euler step (I - nu dt L)^-1 of axisymmetric vorticity diffusion."""

    def __init__(self, time_step, kinematic_viscosity, grid_size_r, grid_size_z, dx,
                 real_dtype=np.float64, device=None, refine=1):
        self.time_step = time_step
        self.nu_times_dt = time_step * kinematic_viscosity
        self.dx = dx
        self.grid_size_r = grid_size_r
        self.grid_size_z = grid_size_z
        self.real_dtype = real_dtype
        self.radial_coord = radial_coord(dx, grid_size_r)
        r = self.radial_coord
        nr, nz = grid_size_r, grid_size_z
        inv_dx2 = 1 / dx / dx
        inv_2dx = 1 / 2 / dx
        pz = tridiag(nz, inv_dx2, -2 * inv_dx2, inv_dx2)
        pr = tridiag(nr, inv_dx2, -2 * inv_dx2, inv_dx2)
        npr = tridiag(nr, -inv_2dx, 0.0, inv_2dx) / r - np.identity(nr) / (r ** 2)
        vr, er = eig_sorted_desc(pr + npr)
        vz, ez = eig_sorted_desc(pz)
        spectrum = 1.0 - self.nu_times_dt * (vz.reshape(1, nz) + vr.reshape(nr, 1))
        precision = "f32" if np.dtype(real_dtype) == np.float32 else "f64"
        # the operator inverted: (I - nu dt A_r) (x) I + I (x) (-nu dt A_z)
        self.engine = FastDiagonalisationEngine(
            vr, er, vz, ez, spectrum, row_weight=None, device=device, precision=precision,
            op_r=np.identity(nr) - self.nu_times_dt * (pr + npr), op_z=-self.nu_times_dt * pz,
            refine=refine)

    def step(self, vorticity_field, dt):
        """Performs an implicit Euler timestep for diffusion in axisym
        coordinates, in place. dt must equal the construction time step."""
        if dt != self.time_step:
            raise ValueError(
                "dt should be constant throughout the simulation if using "
                "implicit diffusion! Please use the value of dt being used "
                "to initialize the implicit diffusion stepper"
            )
        self.engine.transform(vorticity_field, vorticity_field)
