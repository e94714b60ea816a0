/*
 * axisym_gb300.h - C ABI of the GB300 (sm_103a) implementation of the
 * PyAxisymFlow per-timestep grid hot path.
 *
 * Conventions
 *   - Every field is a dense row-major (nr, nz) array in device memory:
 *     axis 0 is r (grid_size_r rows), axis 1 is z (grid_size_z, contiguous),
 *     exactly the numpy layout the reference kernels take.
 *   - "_f64" entry points compute in double, "_f32" in float.
 *   - Every call is asynchronous on `stream` (a cudaStream_t; NULL = legacy
 *     default stream) unless its comment says it synchronises.
 *   - Every call returns an axi_status; axi_last_error() describes the last
 *     failure on the calling thread. Nothing allocates device memory unless
 *     its comment says so: scratch is passed in by the caller.
 *   - Citations name the reference function each entry replaces
 *     (file:line, relative to the PyAxisymFlow project root).
 */
#ifndef AXISYM_GB300_H
#define AXISYM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  AXI_OK = 0,
  AXI_ERR_INVALID = 1,        /* bad size, null pointer or parameter */
  AXI_ERR_CUDA = 2,           /* launch or runtime failure */
  AXI_ERR_NOT_CONVERGED = 3,  /* iteration cap reached (least-squares front marching) */
  AXI_ERR_NONFINITE = 4,      /* a NaN/Inf was detected in a reduction */
  AXI_ERR_RANGE = 5           /* a stencil would read outside the grid */
} axi_status;

/* Library version (major * 10000 + minor * 100 + patch). */
int axi_version(void);
/* Message of the last failing call on this thread ("" if none). */
const char* axi_last_error(void);

/* ---------------------------------------------------------------------
 * Velocity from the Stokes stream function.
 * kernels/compute_velocity_from_psi.py:4-17 compute_velocity_from_psi_unb(u_z, u_r, psi, R, dx)
 * ------------------------------------------------------------------ */
int axi_velocity_from_psi_unb_f64(double* u_z, double* u_r, const double* psi, const double* R,
                                  int nr, int nz, double dx, void* stream);
int axi_velocity_from_psi_unb_f32(float* u_z, float* u_r, const float* psi, const float* R,
                                  int nr, int nz, float dx, void* stream);
/* kernels/compute_velocity_from_psi.py:20-34 (_periodic): exchanges `ghost` periodic
 * z-ghost columns of psi in place first (kernels/periodic_boundary_ghost_comm.py:9-13). */
int axi_velocity_from_psi_periodic_f64(double* u_z, double* u_r, double* psi, const double* R,
                                       int nr, int nz, double dx, int ghost, void* stream);
int axi_velocity_from_psi_periodic_f32(float* u_z, float* u_r, float* psi, const float* R,
                                       int nr, int nz, float dx, int ghost, void* stream);

/* ---------------------------------------------------------------------
 * Vorticity from velocity on the interior [1:-1, 1:-1].
 * kernels/compute_vorticity_from_velocity.py:4-13 (_unb) and :16-28 (_periodic,
 * which first exchanges the ghosts of u_r and u_z in place).
 * ------------------------------------------------------------------ */
int axi_vorticity_from_velocity_unb_f64(double* vort, const double* u_z, const double* u_r,
                                        int nr, int nz, double dx, void* stream);
int axi_vorticity_from_velocity_unb_f32(float* vort, const float* u_z, const float* u_r,
                                        int nr, int nz, float dx, void* stream);
int axi_vorticity_from_velocity_periodic_f64(double* vort, double* u_z, double* u_r,
                                             int nr, int nz, double dx, int ghost, void* stream);
int axi_vorticity_from_velocity_periodic_f32(float* vort, float* u_z, float* u_r,
                                             int nr, int nz, float dx, int ghost, void* stream);

/* ---------------------------------------------------------------------
 * Implicit Brinkman penalisation, elementwise over n cells.
 * kernels/brinkmann_penalize.py:4-16
 * brinkmann_penalize(lam, dt, char_func, U_z, U_r, grid_u_z, grid_u_r, penalized_u_z, penalized_u_r)
 * ------------------------------------------------------------------ */
int axi_brinkmann_penalize_f64(double lam, double dt, const double* char_func, double U_z,
                               double U_r, const double* grid_u_z, const double* grid_u_r,
                               double* penalized_u_z, double* penalized_u_r, int64_t n,
                               void* stream);
int axi_brinkmann_penalize_f32(float lam, float dt, const float* char_func, float U_z, float U_r,
                               const float* grid_u_z, const float* grid_u_r, float* penalized_u_z,
                               float* penalized_u_r, int64_t n, void* stream);

/* ---------------------------------------------------------------------
 * Smoothed Heaviside of a level set, elementwise over n cells (reads H).
 * kernels/smooth_Heaviside.py:5-14 smooth_Heaviside(H, phi, blend_w)
 * ------------------------------------------------------------------ */
int axi_smooth_heaviside_f64(double* H, const double* phi, double blend_w, int64_t n,
                             void* stream);
int axi_smooth_heaviside_f32(float* H, const float* phi, float blend_w, int64_t n, void* stream);

/* ---------------------------------------------------------------------
 * Sine taper of boundary vorticity.
 * kernels/kill_boundary_vorticity_sine.py:4-14 (_z, uses Z) and :17-27 (_r, uses R).
 * The reference's literal "1 - Z" / "1 - R" (unit domain length) is kept.
 * ------------------------------------------------------------------ */
int axi_kill_boundary_vorticity_sine_z_f64(double* vort, const double* Z, int nr, int nz,
                                           int width, double dx, void* stream);
int axi_kill_boundary_vorticity_sine_z_f32(float* vort, const float* Z, int nr, int nz,
                                           int width, float dx, void* stream);
int axi_kill_boundary_vorticity_sine_r_f64(double* vort, const double* R, int nr, int nz,
                                           int width, double dx, void* stream);
int axi_kill_boundary_vorticity_sine_r_f32(float* vort, const float* R, int nr, int nz,
                                           int width, float dx, void* stream);

/* ---------------------------------------------------------------------
 * Explicit two-stage diffusion of vorticity.
 * kernels/diffusion_RK2.py:4-44 diffusion_RK2_unb(vorticity, temp_vorticity, R, nu, dt, dx)
 * and :47-89 (_periodic: ghost exchange of vorticity, then of temp_vorticity).
 * temp_vorticity is both scratch and output, as in the reference.
 * ------------------------------------------------------------------ */
int axi_diffusion_rk2_unb_f64(double* vort, double* temp_vort, const double* R, int nr, int nz,
                              double nu, double dt, double dx, void* stream);
int axi_diffusion_rk2_unb_f32(float* vort, float* temp_vort, const float* R, int nr, int nz,
                              float nu, float dt, float dx, void* stream);
int axi_diffusion_rk2_periodic_f64(double* vort, double* temp_vort, const double* R, int nr,
                                   int nz, double nu, double dt, double dx, int ghost,
                                   void* stream);
int axi_diffusion_rk2_periodic_f32(float* vort, float* temp_vort, const float* R, int nr, int nz,
                                   float nu, float dt, float dx, int ghost, void* stream);

/* ---------------------------------------------------------------------
 * Periodic z-ghost exchange, in place.
 * kernels/periodic_boundary_ghost_comm.py:4-15 (plain) and :18-33 (eta: +/- shift
 * of z_max - 2*ghost*dx).
 * ------------------------------------------------------------------ */
int axi_periodic_ghost_comm_f64(double* field, int nr, int nz, int ghost, void* stream);
int axi_periodic_ghost_comm_f32(float* field, int nr, int nz, int ghost, void* stream);
int axi_periodic_ghost_comm_eta_f64(double* field, int nr, int nz, int ghost, double z_max,
                                    double dx, void* stream);
int axi_periodic_ghost_comm_eta_f32(float* field, int nr, int nz, int ghost, float z_max,
                                    float dx, void* stream);

/* ---------------------------------------------------------------------
 * Body force integrals, accumulated in double whatever the field type.
 * kernels/compute_forces.py:4-17 compute_force_on_body(...) -> (F_pen, F_un)
 * kernels/force_projection.py:5-15 force_projection(...) -> (U_z, U_r)
 * `out` is device memory for 2 doubles. `partials` is device scratch of
 * axi_reduction_scratch_doubles(n) doubles. The reduction order is fixed, so
 * repeated calls give identical bits.
 * ------------------------------------------------------------------ */
int64_t axi_reduction_scratch_doubles(int64_t n);
int axi_compute_force_on_body_f64(const double* R, const double* char_func, double rho_f,
                                  double brink_lam, const double* u_z, double U_z_cm_part,
                                  double part_vol, double dt, double diff, int64_t n,
                                  double* partials, double* out, void* stream);
int axi_compute_force_on_body_f32(const float* R, const float* char_func, double rho_f,
                                  double brink_lam, const float* u_z, double U_z_cm_part,
                                  double part_vol, double dt, double diff, int64_t n,
                                  double* partials, double* out, void* stream);
int axi_force_projection_f64(double rho_s, const double* char_func, const double* u_z,
                             const double* u_r, const double* R, int64_t n, double* partials,
                             double* out, void* stream);
int axi_force_projection_f32(double rho_s, const float* char_func, const float* u_z,
                             const float* u_r, const float* R, int64_t n, double* partials,
                             double* out, void* stream);

/* ---------------------------------------------------------------------
 * ENO3 Euler-forward advection with the axis mirror done by index reflection
 * (no doubled buffers). `scratch` is one (nr, nz) field per advected field.
 * kernels/advect_vorticity_via_eno3.py:8-44 (vorticity odd, u_z even, u_r odd;
 *   conservative flux pyst_kernels/advection_flux.py:9-163, step
 *   pyst_kernels/advection_timestep.py:37-54), :47-91 (_periodic: ghost
 *   exchange of u_z, u_r, vorticity first).
 * elasto_kernels/advect_refmap_via_eno3.py:8-54 (eta1 even, eta2 odd, the
 *   non-conservative flux advection_flux.py:166-332), :57-115 (_periodic:
 *   u_z, u_r, eta2 plain exchange; eta1 shifted exchange with z_max).
 * ------------------------------------------------------------------ */
int axi_advect_vorticity_eno3_f64(double* vort, const double* u_z, const double* u_r,
                                  double* scratch, int nr, int nz, double dt_by_dx,
                                  void* stream);
int axi_advect_vorticity_eno3_f32(float* vort, const float* u_z, const float* u_r,
                                  float* scratch, int nr, int nz, float dt_by_dx, void* stream);
int axi_advect_vorticity_eno3_periodic_f64(double* vort, double* u_z, double* u_r,
                                           double* scratch, int nr, int nz, double dt_by_dx,
                                           int ghost, void* stream);
int axi_advect_vorticity_eno3_periodic_f32(float* vort, float* u_z, float* u_r, float* scratch,
                                           int nr, int nz, float dt_by_dx, int ghost,
                                           void* stream);
int axi_advect_refmap_eno3_f64(double* eta1, double* eta2, const double* u_z, const double* u_r,
                               double* scratch2, int nr, int nz, double dt_by_dx, void* stream);
int axi_advect_refmap_eno3_f32(float* eta1, float* eta2, const float* u_z, const float* u_r,
                               float* scratch2, int nr, int nz, float dt_by_dx, void* stream);
int axi_advect_refmap_eno3_periodic_f64(double* eta1, double* eta2, double* u_z, double* u_r,
                                        double* scratch2, int nr, int nz, double dt_by_dx,
                                        int ghost, double z_max, double dx, void* stream);
int axi_advect_refmap_eno3_periodic_f32(float* eta1, float* eta2, float* u_z, float* u_r,
                                        float* scratch2, int nr, int nz, float dt_by_dx,
                                        int ghost, float z_max, float dx, void* stream);

/* ---------------------------------------------------------------------
 * Neo-Hookean solid stress and its curl into vorticity.
 * elasto_kernels/solid_sigma.py:4-29 solid_sigma(s11, s12, s22, G, dx, eta_1, eta_2,
 *   eta_1z, eta_1r, eta_2z, eta_2r): the gradient arrays are outputs written where
 *   the reference writes them; stress uses whatever they hold elsewhere.
 * elasto_kernels/div_tau.py:4-34 update_vorticity_from_solid_stress(vorticity, tau_z,
 *   tau_r, tau11, tau12, tau22, R, dt, dx)
 * ------------------------------------------------------------------ */
int axi_solid_sigma_f64(double* s11, double* s12, double* s22, double G, double dx,
                        const double* eta1, const double* eta2, double* eta1z, double* eta1r,
                        double* eta2z, double* eta2r, int nr, int nz, void* stream);
int axi_solid_sigma_f32(float* s11, float* s12, float* s22, float G, float dx, const float* eta1,
                        const float* eta2, float* eta1z, float* eta1r, float* eta2z,
                        float* eta2r, int nr, int nz, void* stream);
int axi_update_vorticity_from_solid_stress_f64(double* vort, double* tau_z, double* tau_r,
                                               const double* tau11, const double* tau12,
                                               const double* tau22, const double* R, int nr,
                                               int nz, double dt, double dx, void* stream);
int axi_update_vorticity_from_solid_stress_f32(float* vort, float* tau_z, float* tau_r,
                                               const float* tau11, const float* tau12,
                                               const float* tau22, const float* R, int nr,
                                               int nz, float dt, float dx, void* stream);

/* ---------------------------------------------------------------------
 * Least-squares front-marching extrapolation of (eta_x, eta_y), first order.
 * core/src/extrapolate_using_least_squares.hpp:450-467 (impl :142-446) as bound by
 * core/src/extrapolate_using_least_squares_bind.cpp:88-91
 * extrapolate_using_least_squares_till_first_order(current_flag, target_flag, eta_x,
 * eta_y, grid_x, grid_y), int16 flags, double fields, all (n0, n1) row-major.
 * current_flag is updated in place. `work` is device scratch of
 * axi_lsq_work_bytes(n0, n1) bytes. Runs at most max_sweeps sweeps
 * (AXI_ERR_NOT_CONVERGED past it); a 3x3 window leaving the grid gives
 * AXI_ERR_RANGE (the reference reads out of bounds there). Synchronises the
 * stream to return the status; *sweeps_out (host) receives the sweep count.
 * ------------------------------------------------------------------ */
int64_t axi_lsq_work_bytes(int n0, int n1);
int axi_extrapolate_lsq_first_order_f64(int16_t* current_flag, const int16_t* target_flag,
                                        double* eta_x, double* eta_y, const double* grid_x,
                                        const double* grid_y, int n0, int n1, int max_sweeps,
                                        void* work, int* sweeps_out, void* stream);
/* ------------------------------------------------------------------
 * Particle remeshing (kernels/advect_particle.py:5-68)
 *
 * axi_particles_to_mesh_2d_mp4_f64 replaces the compiled
 * pyaxisymflow.core.particles_to_mesh functions particles_to_mesh_2D_mp4
 * (periodic = 1, core/src/particles_to_mesh.hpp:69-91) and
 * particles_to_mesh_2D_unbounded_mp4 (periodic = 0, :163-184): the MP4
 * interpolation of particle values (n0, n1) onto the cell-centred (n0, n1)
 * mesh of spacing dx, dy, bit-identical to the reference's sequential sum.
 * Particle (j, i) must lie less than one cell from mesh point (j, i) along
 * each axis (the reference's remeshing resets particles to the mesh each
 * step); otherwise the output is invalid and axi_p2m_status reports it.
 * `work` is device scratch of axi_p2m_mp4_work_bytes(n0, n1) bytes; both
 * sides 5 .. 65535.
 * ------------------------------------------------------------------ */
int64_t axi_p2m_mp4_work_bytes(int n0, int n1);
int axi_particles_to_mesh_2d_mp4_f64(const double* particle_positions_x,
                                     const double* particle_positions_y,
                                     const double* input_field_at_particle_positions,
                                     double* output_field_at_mesh, int n0, int n1, double dx,
                                     double dy, int periodic, void* work, void* stream);
/* axi_mesh_to_particles_2d_mp4_f64 replaces mesh_to_particles_2D_mp4
 * (periodic = 1) and mesh_to_particles_2D_unbounded_mp4 (periodic = 0) of the
 * compiled pyaxisymflow.core.mesh_to_particles
 * (core/src/mesh_to_particles.hpp, core/src/interpolation/mesh_to_particles_2D.hpp):
 * two mesh fields (n0, n1) interpolated with the MP4 kernel at the particle
 * positions (p0, p1), bit-identical to the reference. */
int axi_mesh_to_particles_2d_mp4_f64(const double* input_field_x, const double* input_field_y,
                                     int n0, int n1, const double* particle_positions_x,
                                     const double* particle_positions_y, double* output_field_x,
                                     double* output_field_y, int p0, int p1, double dx, double dy,
                                     int periodic, void* stream);
/* *displaced (host) = 1 when the last interpolation using `work` met a
 * particle a cell or more from its mesh point (result invalid). Synchronises. */
int axi_p2m_status(const void* work, int n0, int n1, int* displaced, void* stream);
/* kernels/advect_particle.py:20-28: particles on the mirrored (2 nr, nz)
 * domain move by u dt (rows below the axis: u_z even, u_r odd) and take the
 * vorticity (rows below the axis odd). u_z, u_r, vorticity are (nr, nz). */
int axi_advect_particles_prepare_f64(double* z_particles, double* r_particles,
                                     double* vort_particles, const double* vorticity,
                                     const double* u_z, const double* u_r, int nr, int nz,
                                     double dt, void* stream);
/* ---------------------------------------------------------------------
 * Level-set reinitialisation: the signed distance to the zero contour of phi
 * (nr, nz, spacing dx) within `narrow`, the role of
 * skfmm.distance(phi, dx=dx, narrow=narrow) at
 * examples/SoftSphereStreaming/soft_sphere_streaming.py:197. The contour is
 * the marching-squares reconstruction of phi (crossings linearly
 * interpolated on cell edges); points within `narrow` of it get the exact
 * distance to it, with the sign of phi, and in_band = 1; the others keep
 * phi and get in_band = 0 (the reference's masked points, restored from the
 * previous values at :198-199). in_band may be NULL. `out` must not alias
 * `phi`; `work` is device scratch of axi_level_set_work_bytes(nr, nz) bytes;
 * the band is at most 4096 cells wide.
 * ------------------------------------------------------------------ */
int64_t axi_level_set_work_bytes(int nr, int nz);
int axi_level_set_distance_f64(double* out, const double* phi, int nr, int nz, double dx,
                               double narrow, unsigned char* in_band, void* work, void* stream);
/* elasto_kernels/extrapolate_eta_using_least_squares_unb.py:7-30 with
 * elasto_kernels/extrapolate_using_least_squares.py:33-38 folded in: builds the
 * axis-mirrored (2*nr, nz) level set, masked eta and flags (phi < 0, phi <
 * extrap_zone) from the upper-half fields, extrapolates, and copies back.
 * inside_solid is a byte mask (numpy bool). The doubled buffers are caller
 * scratch of 2*nr*nz doubles each; flags of 2*nr*nz int16 each. grid_y must
 * hold 2*nr coordinates (the reference passes z). */
int axi_extrapolate_eta_with_least_squares_f64(
    const uint8_t* inside_solid, const double* ball_phi, double* eta1, double* eta2,
    double* ball_phi_double, double* eta1_double, double* eta2_double, int16_t* current_flag,
    int16_t* target_flag, double extrap_zone, int nr, int nz, const double* grid_x,
    const double* grid_y, int max_sweeps, void* work, int* sweeps_out, void* stream);

/* ---------------------------------------------------------------------
 * Fast-diagonalisation spectral transform (Stokes / potential solve,
 * implicit diffusion step):
 *   out = Er * ((Er_inv_w * in * EzinvT) .* inv_eig) * EzT
 * kernels/FastDiagonalisationStokesSolver.py:130-156 (Er_inv_w = E_r^-1 diag(r)),
 * kernels/FastDiagonalisationPotentialSolver.py:119-145 and
 * kernels/implicit_diffusion_solver.py:108-143 (Er_inv_w = E_r^-1).
 * Er, Er_inv_w: (nr, nr); EzinvT, EzT: (nz, nz); inv_eig: (nr, nz), all
 * row-major double in device memory, from the host eigendecomposition.
 * `in` and `out` are (nr, nz) with row strides ld_in / ld_out >= nz (the
 * periodic examples solve on the ghost-free slice field[:, g:-g]).
 * work: device scratch of 2*nr*nz doubles. `out` may alias `in`.
 * ------------------------------------------------------------------ */
int axi_fd_transform_f64(double* out, int ld_out, const double* in, int ld_in,
                         const double* Er_inv_w, const double* EzinvT, const double* inv_eig,
                         const double* Er, const double* EzT, double* work, int nr, int nz,
                         void* stream);
/* FP32 GEMM on the tcgen05 tensor cores with 3xTF32 split products (FP32
 * accuracy): C (M, N) = A (M, K) * B (N, K)^T, all row-major float, K a
 * multiple of 4. work: device scratch of axi_tf32x3_gemm_work_bytes(M, N, K)
 * bytes. Synchronises the stream (reads the kernel's pipeline status).
 * The operand form of the spectral products in the FP32 engine. */
int64_t axi_tf32x3_gemm_work_bytes(int M, int N, int K);
int axi_tf32x3_gemm(float* C, const float* A, const float* B, int M, int N, int K, void* work,
                    void* stream);
/* ---------------------------------------------------------------------
 * Spectral transform on the tcgen05 tensor cores (FP32 operands, 3xTF32
 * products, FP32 accumulation): the same transform as axi_fd_transform_f64
 * for any boundary-condition set, used by the FP32 solvers
 * (kernels/FastDiagonalisationStokesSolver.py:130-156 and
 * FastDiagonalisationPotentialSolver.py:119-145 with real_dtype float32).
 * Operands are K-major row-major float; every basis matrix is given as a
 * TF32 hi part and its TF32-rounded remainder (lo). nr and nz multiples of 4.
 * ------------------------------------------------------------------ */
typedef struct axi_tc_transform {
  int32_t nr, nz;
  const float* basis[8]; /* E_z^-1 hi, lo (nz, nz); E_r^-1 W hi, lo (nr, nr);
                            E_z hi, lo (nz, nz); E_r hi, lo (nr, nr) */
  const float* inv_eig;  /* (nr, nz) */
  float* in_hi;          /* (nr, nz) split input (axi_tc_split_*) */
  float* in_lo;
  float* work[4];        /* X hi, lo (nz, nr); Y hi, lo (nr, nz) */
  float* out;            /* (nr, nz) */
} axi_tc_transform;

typedef struct axi_tc_plan_info {
  int32_t n;             /* transforms in the plan */
  int32_t n_tiles[4];    /* 128 x 128 output tiles per product stage */
  int32_t reserved;
  int64_t bytes;         /* device bytes of the plan */
} axi_tc_plan_info;

/* Plans n transforms (tensor maps encoded on the host). With plan_dev NULL
 * only fills `info` (size query); else writes the plan (info->bytes) and
 * synchronises the stream. */
int axi_tc_transform_plan(const axi_tc_transform* t, int n, void* plan_dev,
                          axi_tc_plan_info* info, void* stream);
/* Runs every transform of the plan (four grouped tensor-core launches). */
int axi_tc_transform_run(const axi_tc_plan_info* info, const void* plan_dev, void* stream);
/* Pipeline status of the plan's launches (0 = healthy); synchronises. */
int axi_tc_transform_status(const axi_tc_plan_info* info, const void* plan_dev, int* tc_error,
                            void* stream);
/* TF32 split of n values: hi = nearest TF32 value of fl32(x), lo = nearest
 * TF32 value of the remainder x - hi (taken in float, or in double for the
 * f64 form). */
int axi_tc_split_f32(float* hi, float* lo, const float* x, int64_t n, void* stream);
int axi_tc_split_f64(float* hi, float* lo, const double* x, int64_t n, void* stream);
/* Residual of one refinement step, in FP64: res = rhs - (L psi) / w_i with
 * L = A_r (x) I + I (x) A_z the discrete operator and w the row weight
 * (the solver solves L psi = diag(w) rhs; its transform applies w itself,
 * so the residual it is given is unweighted). ar, az
 * hold the sub, main and super diagonal of each row (3 nr, 3 nz doubles);
 * wrap0 = A_z[0, nz-1], wrap1 = A_z[nz-1, 0] (periodic z, else 0);
 * row_weight may be NULL (w = 1). */
int axi_fd_residual_f64(double* res, const double* rhs, const double* psi,
                        const double* row_weight, const double* ar, const double* az, int nr,
                        int nz, double wrap0, double wrap1, void* stream);
/* y += x and y = x (float -> double), n values. */
int axi_add_f32_to_f64(double* y, const float* x, int64_t n, void* stream);
int axi_widen_f32_to_f64(double* y, const float* x, int64_t n, void* stream);

/* Allocation-free form of axi_fd_transform_f64 (no counterpart in the
 * reference). For callers that cannot call cudaMalloc: a host whose device
 * memory is owned by another allocator. The two intermediate products live in
 * a device array inside this library, sized for
 * nr * nz <= axi_fd_transform_static_max_cells() (512 x 1024 cells, 8 MiB,
 * resident on every GPU that loads the library until the process exits);
 * larger grids are rejected with AXI_ERR_INVALID. The first call in a context
 * looks up the array's device address (with that device current). All calls
 * share the array, so calls that overlap on the GPU (other streams, other
 * host threads) race; serialise them on one stream. Nothing is allocated or
 * freed. */
int64_t axi_fd_transform_static_max_cells(void);
int axi_fd_transform_static_f64(double* out, int ld_out, const double* in, int ld_in,
                                const double* Er_inv_w, const double* EzinvT,
                                const double* inv_eig, const double* Er, const double* EzT,
                                int nr, int nz, void* stream);
/* Row-major double GEMM C = A(M,K) * B(K,N) (.* S(M,N) if S != NULL), row
 * strides ldc, lda, ldb; S is dense (row stride N). */
int axi_dgemm_f64(double* C, int ldc, const double* A, int lda, const double* B, int ldb,
                  const double* S, int M, int N, int K, void* stream);

/* ---------------------------------------------------------------------
 * Fused per-timestep engine for flows past rigid bodies, many cases per launch.
 * One step = the loop body of examples/FlowPastSphere/flow_past_sphere.py:107-188
 * (kill_boundary_vorticity_sine_z/_r, FastDiagonalisationStokesSolver.solve,
 * compute_velocity_from_psi_unb, free stream ramp, CFL dt,
 * brinkmann_penalize + compute_vorticity_from_velocity_unb, drag,
 * advect_vorticity_via_eno3, diffusion_RK2_unb) for every case of a plan.
 * dt, the drag coefficient and the simulated time stay on the device (state
 * block), so steps never synchronise with the host and can be captured in a
 * CUDA graph. Non-finite velocity or drag sets bit AXI_ERR_NONFINITE in the
 * AXI_ST_STATUS word of the case.
 * ------------------------------------------------------------------ */
/* Words of the per-case device state block (doubles). */
enum {
  AXI_ST_T = 0,        /* simulated time */
  AXI_ST_DT = 1,       /* time step of the current / last step */
  AXI_ST_CD = 2,       /* drag coefficient of the last step */
  AXI_ST_STEPS = 3,    /* steps taken */
  AXI_ST_UMAX = 4,     /* bits of max(|u_z| + |u_r|) of the current step (uint64) */
  AXI_ST_COUNT = 5,    /* tile counters of the current step (two uint32) */
  AXI_ST_STATUS = 6,   /* sticky axi_status bits (uint32 in the low word) */
  AXI_ST_FORCE = 7,    /* last sum of r chi u_z over the grid (FP64) */
  AXI_ST_UFREE = 8,    /* free stream of the current step, U0 * ramp(t) */
  AXI_ST_LAMDT = 9,    /* lam * dt */
  AXI_ST_ADV = 10,     /* -dt / dx (ENO3 flux factor) */
  AXI_ST_C1 = 11,      /* 0.5 nu dt (RK2 stage 1) */
  AXI_ST_C2 = 12,      /* nu dt (RK2 stage 2) */
  AXI_ST_ZCM = 13,     /* sedimenting body: centre z */
  AXI_ST_UBODY = 14,   /* sedimenting body: velocity along z */
  AXI_ST_DIFF = 15,    /* sedimenting body: last velocity increment (unsteady force) */
  AXI_ST_FTOTAL = 16,  /* sedimenting body: last total force */
  AXI_ST_F32 = 17,     /* words 17-23: float copies of the step scalars that
                          the float engine's per-cell code reads (internal) */
  AXI_ST_WORDS = 24
};

enum { AXI_CASE_SEDIMENTING = 1 };

/* Stencil tiles of the engine: AXI_TILE_NR rows x AXI_TILE_NZ columns. A
 * case has ceil(nr / AXI_TILE_NR) * ceil(nz / AXI_TILE_NZ) of them. */
enum { AXI_TILE_NR = 32, AXI_TILE_NZ = 64 };

/* One flow-past-rigid-body case. Fields are (nr, nz) row-major in the engine
 * precision (double for _f64, float for _f32); rinv2dx, rinv2 and rw are
 * per-row vectors (length nr) and zw a per-column vector (length nz) in the
 * engine precision; r and z are double vectors of length nr and nz. partials
 * holds 2 doubles per stencil tile of the case. nr * nz < 2^31. */
typedef struct axi_case {
  int32_t nr, nz;
  int32_t kill_width;
  int32_t stencil_tile0; /* first stencil tile of this case in the plan */
  double dx, nu, lam, U0, t_ramp, cfl, U_body, cd_scale, dt_diff, eps;
  double inv_dx2, inv_2dx;
  /* AXI_CASE_SEDIMENTING: a rigid sphere of radius r_body falling along z
   * (examples/SedimentingRigidSphere/falling_rigid_sphere.py:136-181): the
   * Brinkman target is the body velocity, the force integral and the body ODE
   * run on the device in FP64 and the mask is rebuilt every step. */
  int32_t flags;
  int32_t pad0;
  double rho_f, rho_s, grav, part_mass, part_vol, r_body, blend_w;
  void* omega;
  void* psi;
  void* u_z;
  void* u_r;
  void* chi;
  const double* kill_coef; /* 3 * kill_width sine-taper factors: z start, z end, outer r */
  const double* r;
  const double* z;
  const void* rinv2dx;   /* 1 / (2 dx r_i) */
  const void* rinv2;     /* 1 / r_i^2 */
  const void* rw;        /* r_i (drag weight) */
  const void* zw;        /* z_j */
  const void* Er;        /* (nr, nr) */
  const void* Er_inv_w;  /* (nr, nr), E_r^-1 diag(r) */
  const void* EzinvT;    /* (nz, nz) */
  const void* EzT;       /* (nz, nz) */
  const void* inv_eig;   /* (nr, nz) */
  void* gemm_work;       /* 2 nr nz: spectral-solve scratch, then the penalised omega */
  double* state;         /* AXI_ST_WORDS doubles */
  double* partials;      /* one double per stencil tile of the case */
  double* history;       /* optional: 2 doubles (dt, Cd) per step, or NULL */
  int64_t history_len;
  /* FP32 engine with the spectral products on the tensor cores (plan flag
   * AXI_PLAN_TENSOR_CORES): TF32 hi parts and TF32 remainders (lo) of the
   * operands, row-major float. */
  void* omega_hi;        /* (nr, nz), kept in step with omega */
  void* omega_lo;
  const void* tc_basis[8]; /* E_z^-1 hi, lo (nz, nz); E_r^-1 diag(r) hi, lo (nr, nr);
                              E_z hi, lo (nz, nz); E_r hi, lo (nr, nr) */
  void* tc_work[4];        /* X hi, lo (nz, nr); Y hi, lo (nr, nz) */
  /* AXI_PLAN_DCT_Z: tables of the z transform for this nz (shared by cases of
   * equal nz), float for the float engine and double for the double engine:
   * exp(-2 pi i m / nz) as (cos, sin) pairs, m < nz;
   * (cos, sin)(pi k / 2 nz), k < nz; c_k; 1 / c_k (c_0 = sqrt(1 / nz),
   * c_k = sqrt(2 / nz)); inv_eig then holds 1 / (lambda_r_i + lambda_z_k) in
   * DCT order, lambda_z_k = (2 - 2 cos(pi k / nz)) / dx^2. */
  const void* dct_table;
  /* AXI_PLAN_REFINE: the low part of psi, float (nr, nz): psi is carried as
   * the pair psi + psi_lo (about 48 significant bits), so the velocity
   * differences of neighbouring psi values keep the refined solve's
   * accuracy instead of the float rounding of psi. Start at zero. */
  void* psi_lo;
} axi_case;

/* Launch choices of a plan that change the scheduling of the work, never its
 * results: every choice gives bit-identical fields (the work units, their
 * arithmetic and every reduction order are fixed; only which block takes which
 * unit, and when, changes). 0 selects the built-in default. Set them in
 * axi_plan_info.tune after axi_plan_init and before axi_plan_upload (the
 * orders are laid out by the upload); the launch choices apply to every
 * later step. No counterpart in the reference (its kernels are pystencils /
 * numpy calls); pyaxisymflow_gb300.autotune picks them per grid-size mix by
 * measurement. */
typedef struct axi_tuning {
  /* resident blocks per SM of vel_max, penalise and advect_diffuse (0: all
   * that fit; penalise and advect_diffuse then take one tile per block) */
  int32_t stencil_blocks_per_sm[3];
  /* L2 prefetch distance of the stencil tiles and the DCT items, in resident
   * waves (0: one wave; -1: no prefetch) */
  int32_t prefetch_waves;
  /* persistent CTAs of the tensor-core products, percent of the SMs (0: 100) */
  int32_t tc_ctas_percent;
  /* tensor-core tile order: 0 longest main loop (K) first, 1 case order */
  int32_t tc_tile_order;
  /* DCT item order: 0 case order with the shortest rows last, 1 case order,
   * 2 longest rows first */
  int32_t dct_item_order;
  int32_t reserved;
} axi_tuning;

/* Launch plan of a set of cases: tile tables in device memory. */
typedef struct axi_plan_info {
  int32_t n_cases;
  int32_t n_stencil_tiles; /* AXI_TILE_NR x AXI_TILE_NZ cell tiles over all cases */
  int32_t n_gemm_tiles;    /* output tiles of the grouped spectral products */
  int32_t elem_bytes;      /* 8: float64 fields, 4: float32 fields */
  int64_t bytes;           /* device bytes the plan needs */
  int32_t flags;           /* AXI_PLAN_* */
  int32_t n_tc_tiles[4];   /* tensor-core tiles per spectral stage */
  int32_t n_dct_items;     /* row groups of the z transforms (AXI_PLAN_DCT_Z) */
  axi_tuning tune;         /* launch choices (zero: defaults) */
} axi_plan_info;

/* AXI_PLAN_DCT_Z: the z-direction products run as orthonormal DCT-II /
 * DCT-III transforms (the eigenbasis of the Neumann z operator); every nz
 * even with no prime factor other than 2 and 3. Float fields (with
 * AXI_PLAN_TENSOR_CORES): the radial products on the tensor cores,
 * omega_hi / omega_lo and the z entries of tc_basis unused (may be NULL).
 * Double fields (without it): the radial products on the SIMT FP64 GEMM,
 * nz <= 2048, dct_table holding the tables in double. */
/* AXI_PLAN_REFINE (with AXI_PLAN_DCT_Z): every solve is one step of
 * iterative refinement started from the psi the case already holds (the
 * previous step's; zero for a new case): the forward z transform reads the
 * residual omega - (A psi) / r of the discrete operator instead of omega, and
 * the last radial product adds its result to the pair (psi, psi_lo), which
 * the velocity kernels read back as psi + psi_lo. The solve error then
 * shrinks with the step-to-step change of psi instead of with psi itself; the
 * first solve of a case is the plain solve. Needs psi_lo. */
enum { AXI_PLAN_TENSOR_CORES = 1, AXI_PLAN_DCT_Z = 2, AXI_PLAN_REFINE = 4 };

/* Host only: validates the cases, assigns each its first tile
 * (cases[k].stencil_tile0) and fills `info` (sizes of the plan). flags:
 * AXI_PLAN_TENSOR_CORES (FP32 only) runs the spectral products as tcgen05
 * 3xTF32 GEMMs (the tc_* and omega_hi / omega_lo members must be set). */
int axi_plan_init(axi_case* cases, int n_cases, int elem_bytes, int flags, axi_plan_info* info);
/* Tensor-core plans: recompute the TF32 operand copy of omega (omega_hi,
 * omega_lo) of every case after the caller overwrote omega. */
int axi_rigid_refresh_operands(const axi_plan_info* info, const void* plan_dev, void* stream);
/* Pipeline status of the plan's asynchronous copies (tensor-core products
 * and the stencil kernels' TMA boxes) since the plan was uploaded: 0 =
 * healthy; 1-4 a tensor-core wait, 5-6 a stencil wait timed out.
 * Synchronises the stream. */
int axi_plan_tc_status(const axi_plan_info* info, const void* plan_dev, int* tc_error,
                       void* stream);
/* Copies the case table and tile tables into plan_dev (caller-allocated,
 * info->bytes); synchronises the stream. Re-upload after changing a case. */
int axi_plan_upload(const axi_case* cases, const axi_plan_info* info, void* plan_dev,
                    void* stream);
/* Advances every case of the plan by n_steps steps (float64 / float32 fields). */
int axi_rigid_step_f64(const axi_plan_info* info, const void* plan_dev, int n_steps,
                       void* stream);
int axi_rigid_step_f32(const axi_plan_info* info, const void* plan_dev, int n_steps,
                       void* stream);
/* One phase of a step (0 kill, 1 spectral transform, 2 velocity max and dt,
 * 3 penalisation and drag, 4 advection and both diffusion stages); running
 * phases 0..4 in order equals one step. Phase 3 leaves the penalised
 * vorticity in the first nr x nz elements of gemm_work (omega unchanged);
 * phase 4 advances it into omega. Phases 5..8 are the four launches of
 * phase 1 one at a time (z product or DCT, radial product, z product or
 * inverse DCT, radial product). Lets a caller time each kernel. */
int axi_rigid_phase_f64(const axi_plan_info* info, const void* plan_dev, int phase,
                        void* stream);
int axi_rigid_phase_f32(const axi_plan_info* info, const void* plan_dev, int phase,
                        void* stream);

/* ---------------------------------------------------------------------
 * Soft-sphere streaming loop with the time step on the device
 * (examples/SoftSphereStreaming/soft_sphere_streaming.py:129-272).
 * The drop-in kernels above take dt and t as host scalars, so a host loop
 * must read max |u| back each step. These entries keep dt and t in a state
 * block of AXI_SOFT_WORDS doubles (zero it before the first step) and read
 * them on the device; the arithmetic is that of the host-dt kernels, so a
 * loop made of them (pyaxisymflow_gb300.simulation.SoftSphereEngine) runs
 * without a host round trip and can be captured in a CUDA graph. FP64.
 * ------------------------------------------------------------------ */
enum {
  AXI_SOFT_T = 0,       /* simulated time */
  AXI_SOFT_DT = 1,      /* time step of the current step */
  AXI_SOFT_STEPS = 2,   /* steps taken */
  AXI_SOFT_STATUS = 3,  /* sticky status bits (uint64 view): 1 << AXI_ERR_* */
  AXI_SOFT_SWEEPS = 4,  /* largest extrapolation sweep count seen */
  AXI_SOFT_UMAX = 5,    /* scratch of axi_soft_dt (kept zero between calls) */
  AXI_SOFT_COUNT = 6,   /* scratch of axi_soft_dt (kept zero between calls) */
  AXI_SOFT_WORDS = 8
};
/* dt = min(dt_elastic, cfl_dx / (max(|u_z| + |u_r|) + eps), dt_diffusive) into
 * state[AXI_SOFT_DT] (soft_sphere_streaming.py:168-172). */
int axi_soft_dt_f64(const double* u_z, const double* u_r, int64_t n, double* state,
                    double dt_elastic, double cfl_dx, double dt_diffusive, double eps,
                    void* stream);
/* ENO3 advection with dt from the state: refmap != 0 advects (eta1, eta2) as
 * axi_advect_refmap_eno3_f64, else f0 = omega as axi_advect_vorticity_eno3_f64
 * (scratch: 2 or 1 fields). */
int axi_soft_advect_eno3_f64(double* f0, double* f1, int refmap, const double* u_z,
                             const double* u_r, double* scratch, int nr, int nz, double dx,
                             const double* state, void* stream);
/* ball_phi = where(ball_phi > band, -sqrt((eta1 - z_cm)^2 + eta2^2) + r_ball, ball_phi)
 * (soft_sphere_streaming.py:191-193; band = -3 dx). */
int axi_soft_pin_level_set_f64(double* ball_phi, const double* eta1, const double* eta2,
                               int64_t n, double z_cm, double r_ball, double band,
                               void* stream);
/* chi = smooth_Heaviside(phi, blend_w) and inside = chi > 0.5 (:205-206). */
int axi_soft_mask_f64(double* chi, uint8_t* inside, const double* phi, int64_t n,
                      double blend_w, void* stream);
/* The extrapolation of axi_extrapolate_eta_with_least_squares_f64 without a
 * host round trip: failures set state[AXI_SOFT_STATUS] bits, the sweep count
 * goes to state[AXI_SOFT_SWEEPS]. */
int axi_soft_extrapolate_eta_f64(const uint8_t* inside_solid, const double* ball_phi,
                                 double* eta1, double* eta2, double* ball_phi_double,
                                 double* eta1_double, double* eta2_double, int16_t* current_flag,
                                 int16_t* target_flag, double extrap_zone, int nr, int nz,
                                 const double* grid_x, const double* grid_y, int max_sweeps,
                                 void* work, double* state, void* stream);
/* sigma_ij *= chi (:236-238). */
int axi_soft_stress_mask_f64(double* s11, double* s12, double* s22, const double* chi,
                             int64_t n, void* stream);
/* axi_update_vorticity_from_solid_stress_f64 with dt from the state (:239-241). */
int axi_soft_update_vorticity_from_solid_stress_f64(double* vort, double* tau_z, double* tau_r,
                                                    const double* t11, const double* t12,
                                                    const double* t22, const double* R, int nr,
                                                    int nz, double dx, const double* state,
                                                    void* stream);
/* Tether mask: smooth_Heaviside(-sqrt((Z - z_cm - e_r_ball sin(omega t))^2 + R^2)
 * + zeta_r_ball, blend_w) with t from the state (:243-245). */
int axi_soft_tether_f64(double* tether_chi, const double* Z, const double* R, int64_t n,
                        const double* state, double z_cm, double e_r_ball, double omega,
                        double zeta_r_ball, double blend_w, void* stream);
/* Brinkman penalisation of (u_z, u_r) towards (U0 cos(omega_f t), 0) with
 * lam dt chi, then omega += curl(u_pen - u) on the interior (:248-264);
 * d_z, d_r: (nr, nz) scratch. */
int axi_soft_penalise_f64(double* omega, double* u_z, double* u_r, const double* tether_chi,
                          double* d_z, double* d_r, int nr, int nz, double dx, double lam,
                          double U0, double omega_f, const double* state, void* stream);
/* axi_diffusion_rk2_unb_f64 with dt from the state (:267). */
int axi_soft_diffusion_rk2_f64(double* vort, double* tmp, const double* R, int nr, int nz,
                               double nu, double dx, const double* state, void* stream);
/* t += dt, steps += 1 (:270-272). */
int axi_soft_advance_f64(double* state, void* stream);

/* ---------------------------------------------------------------------
 * Orthonormal FP64 DCT-II / DCT-III along the rows of a (rows, N) array, for
 * a spectral solve outside the rigid engine whose z operator is the Neumann
 * Laplacian (kernels/FastDiagonalisationStokesSolver.py:41-97): E_z^-1 x is
 * the DCT-II of each row, E_z y the DCT-III (no counterpart in the
 * reference, which multiplies by the dense eigenvector matrices). N even with
 * factors 2 and 3 only, N <= 2048. table: the double tables of the z
 * transform as axi_case.dct_table describes them (6 N doubles).
 * axi_dct64_plan_f64 fills a caller-allocated device plan
 * (axi_dct64_plan_bytes) for fixed in / out arrays and synchronises the
 * stream; axi_dct64_run_f64 transforms with it (no host data: capturable).
 * ------------------------------------------------------------------ */
int64_t axi_dct64_plan_bytes(int rows, int N);
int axi_dct64_plan_f64(const double* in, double* out, int rows, int N, const double* table,
                       int forward, void* plan_dev, void* stream);
int axi_dct64_run_f64(const void* plan_dev, int rows, int N, int forward, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* AXISYM_GB300_H */
