"""Drop-in for pyaxisymflow/kernels/FastDiagonalisationPotentialSolver.py:6-145."""
import numpy as np

from ._spectral import FastDiagonalisationEngine, eig_sorted_desc, radial_coord, tridiag

NEUMANN_ZR = "homogenous_neumann_along_z_and_r"


class FastDiagonalisationPotentialSolver:
    """Solves psi_rr + psi_zz + psi_r / r = rhs by fast diagonalisation."""

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
        pz = tridiag(nz, inv_dx2, -2 * inv_dx2, inv_dx2)
        pr = tridiag(nr, inv_dx2, -2 * inv_dx2, inv_dx2)
        dr = tridiag(nr, -inv_2dx, 0.0, inv_2dx) / self.radial_coord
        if bc_type == NEUMANN_ZR:
            pz[0, 0] = -inv_dx2
            pz[-1, -1] = -inv_dx2
            pr[-1, -1] = -inv_dx2
            dr[-1, -2] = 0
        vr, er = eig_sorted_desc(pr + dr)
        vz, ez = eig_sorted_desc(pz)
        spectrum = vz.reshape(1, nz) + vr.reshape(nr, 1)
        precision = "f32" if np.dtype(real_dtype) == np.float32 else "f64"
        self.engine = FastDiagonalisationEngine(vr, er, vz, ez, spectrum, row_weight=None,
                                                device=device, precision=precision,
                                                op_r=pr + dr, op_z=pz, refine=refine)

    def solve(self, solution_field, rhs_field):
        """solution_field[...] = the potential for rhs_field (CUDA float64)."""
        self.engine.transform(solution_field, rhs_field)
