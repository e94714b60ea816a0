"""Drop-in for pyaxisymflow/kernels/FastDiagonalisationStokesSolver.py:6-156."""
import numpy as np

from ._spectral import FastDiagonalisationEngine, eig_sorted_desc, radial_coord, tridiag

NEUMANN_ZR = "homogenous_neumann_along_z_and_r"
NEUMANN_R_PERIODIC_Z = "homogenous_neumann_along_r_and_periodic_along_z"
DIRICHLET_R_PERIODIC_Z = "homogenous_dirichlet_along_r_and_periodic_along_z"


class FastDiagonalisationStokesSolver:
    """Solves the Stokes stream-function pseudo Poisson
    -psi_rr - psi_zz + psi_r / r = r * omega by fast diagonalisation."""

    def __init__(self, grid_size_r, grid_size_z, dx, real_dtype=np.float64,
                 bc_type=NEUMANN_ZR, device=None, refine=1):
        self.dx = dx
        self.grid_size_r = grid_size_r
        self.grid_size_z = grid_size_z
        self.real_dtype = real_dtype
        self.bc_type = bc_type
        self.radial_coord = radial_coord(dx, grid_size_r)
        nr, nz = grid_size_r, grid_size_z
        inv_dx2 = 1 / dx / dx
        inv_2dx = 1 / 2 / dx
        # construct_fdm_matrices (:41-67)
        pz = tridiag(nz, -inv_dx2, 2 * inv_dx2, -inv_dx2)
        pr = tridiag(nr, -inv_dx2, 2 * inv_dx2, -inv_dx2)
        dr = tridiag(nr, inv_2dx, 0.0, -inv_2dx) / self.radial_coord
        # apply_boundary_conds_to_poisson_matrices (:69-97)
        if bc_type == NEUMANN_ZR:
            pz[0, 0] = inv_dx2
            pz[-1, -1] = inv_dx2
            pr[-1, -1] = inv_dx2
            dr[-1, -2] = 0
        elif bc_type == NEUMANN_R_PERIODIC_Z:
            pz[0, -1] = pz[0, 1]
            pz[-1, 0] = pz[-1, -2]
            pr[-1, -1] = inv_dx2
            dr[-1, -2] = 0
        elif bc_type == DIRICHLET_R_PERIODIC_Z:
            pz[0, -1] = pz[0, 1]
            pz[-1, 0] = pz[-1, -2]
        else:
            raise ValueError(f"unknown bc_type {bc_type!r}")
        # compute_spectral_decomp_of_poisson_matrices (:99-128)
        vr, er = eig_sorted_desc(pr - dr)
        vz, ez = eig_sorted_desc(pz)
        spectrum = vz.reshape(1, nz) + vr.reshape(nr, 1)
        precision = "f32" if np.dtype(real_dtype) == np.float32 else "f64"
        self.engine = FastDiagonalisationEngine(vr, er, vz, ez, spectrum,
                                                row_weight=self.radial_coord.ravel(),
                                                device=device, precision=precision,
                                                op_r=pr - dr, op_z=pz, refine=refine)

    def solve(self, solution_field, rhs_field):
        """solution_field[...] = psi solving the pseudo Poisson for rhs_field.

        real_dtype float64: FP64 products; CUDA float64 tensors, rows may be
        strided (e.g. field[:, g:-g]). real_dtype float32: the products run on
        the tcgen05 tensor cores (3xTF32, FP32 accumulation), followed by
        `refine` steps of iterative refinement with an FP64 residual; fields
        may be float32 or float64 (the refined result is kept in FP64)."""
        self.engine.transform(solution_field, rhs_field)
