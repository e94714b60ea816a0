/*
 * C restatement of the oracle's per-step grid kernels, with OpenMP: the CPU
 * baseline of the rigid and sedimenting sphere loops. TEST / MEASUREMENT
 * INFRASTRUCTURE ONLY: the timed CPU baseline and the checks of this file
 * against the numpy oracle use it; the GPU product never does.
 *
 * The reference runs these kernels as numba-compiled loops
 * (kernels/compute_velocity_from_psi.py:4-17, brinkmann_penalize.py:4-16,
 * compute_vorticity_from_velocity.py:4-13, diffusion_RK2.py:4-44) and its
 * ENO3 advection as pystencils-generated C with OpenMP
 * (pyst_kernels/advection_flux.py:9-163, advection_timestep.py:37-54, driven
 * by kernels/advect_vorticity_via_eno3.py:8-44). Each function below keeps
 * the operation order of the numpy oracle (oracle/kernels.py), so that, built
 * without FMA contraction, it gives the oracle's bits. Rows are split across
 * OpenMP threads; no result depends on the thread count.
 *
 * Fields are row-major (nr, nz) double arrays; R and Rm2 are the (nr, nz)
 * arrays of r and r^-2 that the oracle uses.
 */
#include <math.h>
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void ora_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int ora_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* compute_velocity_from_psi_unb (oracle/kernels.py compute_velocity_from_psi_unb),
 * then u_z += u_add when add_free_stream is set; returns max(|u_z| + |u_r|). */
double ora_velocity_from_psi(double* u_z, double* u_r, const double* psi, const double* R,
                             int nr, int nz, double dx, int add_free_stream, double u_add) {
  const double tdx = 2 * dx;
  double vmax = 0.0;
#pragma omp parallel for schedule(static) reduction(max : vmax)
  for (int i = 0; i < nr; ++i) {
    const double* p = psi + (size_t)i * nz;
    const double* rr = R + (size_t)i * nz;
    double* uz = u_z + (size_t)i * nz;
    double* ur = u_r + (size_t)i * nz;
    for (int j = 0; j < nz; ++j) {
      double v;
      if (i == 0) {
        v = (((-psi[2 * (size_t)nz + j]) + 4 * psi[(size_t)nz + j]) - 3 * psi[j]) / tdx / rr[j];
      } else if (i == nr - 1) {
        v = ((p[j - 2 * (size_t)nz] - 4 * p[j - (size_t)nz]) + 3 * p[j]) / tdx / rr[j];
      } else {
        v = (p[j + (size_t)nz] - p[j - (size_t)nz]) / tdx / rr[j];
      }
      if (add_free_stream) v = v + u_add;
      uz[j] = v;
      double w;
      if (j == 0) {
        w = -(((-p[2]) + 4 * p[1]) - 3 * p[0]) / tdx / rr[0];
      } else if (j == nz - 1) {
        w = -((p[nz - 3] - 4 * p[nz - 2]) + 3 * p[nz - 1]) / tdx / rr[nz - 1];
      } else {
        w = -(p[j + 1] - p[j - 1]) / tdx / rr[j];
      }
      ur[j] = w;
      const double s = fabs(v) + fabs(w);
      if (s > vmax) vmax = s;
    }
  }
  return vmax;
}

/* brinkmann_penalize with target (U_z, 0) into u_z, u_r, then
 * omega += curl(u_pen - u) on the interior (compute_vorticity_from_velocity_unb
 * of the differences, added as the oracle's `w += penal`). d_z, d_r: scratch. */
void ora_penalise(double* omega, double* u_z, double* u_r, const double* chi, int nr, int nz,
                  double lamdt, double U_z, double dx, double* d_z, double* d_r) {
  const double tdx = 2 * dx;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nr; ++i) {
    for (int j = 0; j < nz; ++j) {
      const size_t c = (size_t)i * nz + j;
      const double lc = lamdt * chi[c];
      const double den = 1 + lc;
      const double pz = (u_z[c] + lc * U_z) / den;
      const double pr = (u_r[c] + lc * 0.0) / den;
      d_z[c] = pz - u_z[c];
      d_r[c] = pr - u_r[c];
      u_z[c] = pz;
      u_r[c] = pr;
    }
  }
#pragma omp parallel for schedule(static)
  for (int i = 1; i < nr - 1; ++i) {
    for (int j = 1; j < nz - 1; ++j) {
      const size_t c = (size_t)i * nz + j;
      const double pw = (d_r[c + 1] - d_r[c - 1]) / tdx - (d_z[c + nz] - d_z[c - nz]) / tdx;
      omega[c] = omega[c] + pw;
    }
  }
}

/* ENO3 face value of f*u between cells 0 and 1 (oracle _eno3_face_conservative). */
static inline double face(double fm1, double f0, double f1, double f2, double um1, double u0,
                          double u1, double u2) {
  if (u0 > -u1) return ((1.0 / 3) * f1 * u1 + (5.0 / 6) * f0 * u0) - (1.0 / 6) * fm1 * um1;
  return ((1.0 / 3) * f0 * u0 + (5.0 / 6) * f1 * u1) - (1.0 / 6) * f2 * u2;
}

/* value of a field mirrored about the axis: row -1-k is parity * row k */
static inline double mir(const double* f, int row, int col, int nz, double parity) {
  return row >= 0 ? f[(size_t)row * nz + col] : parity * f[(size_t)(-1 - row) * nz + col];
}

/* advect_vorticity_via_eno3 (oracle gen_advect_vorticity_via_eno3): omega odd,
 * u_z even, u_r odd about the axis; zero flux in the last two rows and the
 * first and last two columns (pystencils ghost layers); `src` receives a copy
 * of omega before the step. */
void ora_advect_eno3(double* omega, const double* u_z, const double* u_r, int nr, int nz,
                     double dt_by_dx, double* src) {
  const double a = -dt_by_dx;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nr; ++i)
    for (int j = 0; j < nz; ++j) src[(size_t)i * nz + j] = omega[(size_t)i * nz + j];
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nr - 2; ++i) {
    for (int j = 2; j < nz - 2; ++j) {
      const double* f = src;
      const double f0 = f[(size_t)i * nz + j];
      const double* fz = f + (size_t)i * nz;
      const double* uz = u_z + (size_t)i * nz;
      const double xf = face(fz[j - 1], f0, fz[j + 1], fz[j + 2], uz[j - 1], uz[j], uz[j + 1],
                             uz[j + 2]);
      const double xb = face(fz[j - 2], fz[j - 1], f0, fz[j + 1], uz[j - 2], uz[j - 1], uz[j],
                             uz[j + 1]);
      const double fm2 = mir(f, i - 2, j, nz, -1.0), fm1 = mir(f, i - 1, j, nz, -1.0);
      const double fp1 = f[(size_t)(i + 1) * nz + j], fp2 = f[(size_t)(i + 2) * nz + j];
      const double um2 = mir(u_r, i - 2, j, nz, -1.0), um1 = mir(u_r, i - 1, j, nz, -1.0);
      const double u0 = u_r[(size_t)i * nz + j];
      const double up1 = u_r[(size_t)(i + 1) * nz + j], up2 = u_r[(size_t)(i + 2) * nz + j];
      const double yf = face(fm1, f0, fp1, fp2, um1, u0, up1, up2);
      const double yb = face(fm2, fm1, f0, fp1, um2, um1, u0, up1);
      double flux = 0.0;
      flux = flux + a * xf;
      flux = flux - a * xb;
      flux = flux + a * yf;
      flux = flux - a * yb;
      omega[(size_t)i * nz + j] = f0 + flux;
    }
  }
}

/* the bracketed operator of diffusion_RK2 at interior cell c (oracle _rk2_operator) */
static inline double rk2_op(const double* w, size_t c, int nz, double dx2, double tdx,
                            double r, double rm2) {
  const double n = w[c + nz], s = w[c - nz], e = w[c + 1], ww = w[c - 1], ce = w[c];
  return ((((n + s) + e) + ww) - 4 * ce) / dx2 + (n - s) / tdx / r - ce * rm2;
}

/* diffusion_RK2_unb (oracle diffusion_RK2_unb); tmp receives the stage-1 field. */
void ora_diffusion_rk2(double* omega, double* tmp, const double* R, const double* Rm2, int nr,
                       int nz, double nu, double dt, double dx) {
  const double dx2 = dx * dx, tdx = 2 * dx;
  const double c1 = 0.5 * nu * dt, c2 = nu * dt;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nr; ++i) {
    for (int j = 0; j < nz; ++j) {
      const size_t c = (size_t)i * nz + j;
      double v = omega[c];
      if (i >= 1 && i < nr - 1 && j >= 1 && j < nz - 1)
        v = v + c1 * rk2_op(omega, c, nz, dx2, tdx, R[c], Rm2[c]);
      tmp[c] = v;
    }
  }
#pragma omp parallel for schedule(static)
  for (int i = 1; i < nr - 1; ++i) {
    for (int j = 1; j < nz - 1; ++j) {
      const size_t c = (size_t)i * nz + j;
      omega[c] = omega[c] + c2 * rk2_op(tmp, c, nz, dx2, tdx, R[c], Rm2[c]);
    }
  }
}

/* The sedimenting body's mask rebuild (oracle sedimenting_step: the level set
 * -sqrt((Z - z_cm)^2 + R^2) + radius, then smooth_Heaviside). */
void ora_sphere_mask(double* chi, const double* Z, const double* R, int nr, int nz, double z_cm,
                     double radius, double w) {
  const double pi = 3.141592653589793;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nr; ++i) {
    for (int j = 0; j < nz; ++j) {
      const size_t c = (size_t)i * nz + j;
      const double dz = Z[c] - z_cm, dr = R[c] - 0.0;
      const double phi = -sqrt(dz * dz + dr * dr) + radius;
      double h = phi >= w ? 1.0 : 0.0;
      if (fabs(phi) < w) h = h + 0.5 * ((1 + phi / w) + sin(pi * phi / w) / pi);
      chi[c] = h;
    }
  }
}
