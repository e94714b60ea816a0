// ENO3 Euler-forward advection on the meridional plane, axis mirror by index
// reflection.
//
// The reference builds (2 nr, nz) buffers whose lower half is the field flipped
// about the axis (with parity +1 or -1), runs four pystencils flux kernels on
// the interior [2:-2, 2:-2] of that buffer and copies the upper half back
// (kernels/advect_vorticity_via_eno3.py:28-42). Only the upper half survives,
// so this kernel evaluates exactly the upper-half cells and reads row -1-k of
// the mirror as parity * row k. Upper-half rows nr-2, nr-1 and columns 0, 1,
// nz-2, nz-1 lie in the pystencils ghost layers: they receive a zero flux.
//
// Each face value is shared by its two cells: the x_back kernel of cell c
// (pyst_kernels/advection_flux.py:61-73) evaluates the same upwind selector
// (u[c] > -u[c-1] is u[c-1] > -u[c]) and the same three products, in the same
// order, as the x_front kernel of cell c-1 (:32-44), so one face routine serves
// both. The flux accumulation keeps the reference's statement order:
// flux = 0; += a F_x_front; -= a F_x_back; += a F_y_front; -= a F_y_back;
// field += flux (pyst_kernels/advection_timestep.py:45-54), a = -dt/dx.
#include "axi_common.cuh"

namespace {

constexpr int BX = 32;
constexpr int BY = 8;

// Conservative face value of f*u between cells 0 and 1 (advection_flux.py:34-43).
template <typename T>
__device__ __forceinline__ T face_cons(T fm1, T f0, T f1, T f2, T um1, T u0, T u1, T u2) {
  const T third = T(1) / T(3), five6 = T(5) / T(6), sixth = T(1) / T(6);
  if (u0 > -u1) {
    T a = rn_add(rn_mul(rn_mul(third, f1), u1), rn_mul(rn_mul(five6, f0), u0));
    return rn_sub(a, rn_mul(rn_mul(sixth, fm1), um1));
  }
  T a = rn_add(rn_mul(rn_mul(third, f0), u0), rn_mul(rn_mul(five6, f1), u1));
  return rn_sub(a, rn_mul(rn_mul(sixth, f2), u2));
}

// Non-conservative face value of f between cells 0 and 1 (advection_flux.py:193-199).
template <typename T>
__device__ __forceinline__ T face_noncons(T fm1, T f0, T f1, T f2, T u0, T u1) {
  const T third = T(1) / T(3), five6 = T(5) / T(6), sixth = T(1) / T(6);
  if (u0 > -u1) return rn_sub(rn_add(rn_mul(third, f1), rn_mul(five6, f0)), rn_mul(sixth, fm1));
  return rn_sub(rn_add(rn_mul(third, f0), rn_mul(five6, f1)), rn_mul(sixth, f2));
}

// Value of a mirrored field at (row, col), row >= -2: rows below the axis are
// parity * row (-1 - row).
template <typename T>
__device__ __forceinline__ T mir(const T* __restrict__ f, int row, int col, int nz, T parity) {
  return row >= 0 ? f[(long long)row * nz + col] : parity * f[(long long)(-1 - row) * nz + col];
}

// One Euler step for NF fields sharing the velocity (u_z even, u_r odd).
// src[k] holds the pre-step copy of field k, dst[k] receives the new values.
template <typename T, int NF, bool CONS>
__global__ void eno3_step_kernel(T* __restrict__ dst0, T* __restrict__ dst1,
                                 const T* __restrict__ src0, const T* __restrict__ src1,
                                 T par0, T par1, const T* __restrict__ uz,
                                 const T* __restrict__ ur, int nr, int nz, T a,
                                 const double* __restrict__ dt_dev, T dx) {
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  if (i >= nr || j >= nz) return;
  // a device-resident time step (the soft-sphere loop): a = -(dt / dx)
  if (dt_dev) a = -rn_div(static_cast<T>(dt_dev[0]), dx);
  const long long c = (long long)i * nz + j;
  const bool interior = (i < nr - 2) && (j >= 2) && (j < nz - 2);
#pragma unroll
  for (int k = 0; k < NF; ++k) {
    const T* __restrict__ src = k == 0 ? src0 : src1;
    T* __restrict__ dst = k == 0 ? dst0 : dst1;
    const T par = k == 0 ? par0 : par1;
    T flux = T(0);
    if (interior) {
      // x direction (z axis): cells j-2 .. j+2 of row i
      const T* row = src + (long long)i * nz;
      const T* vrow = uz + (long long)i * nz;
      const T fm2 = row[j - 2], fm1 = row[j - 1], f0 = row[j], f1 = row[j + 1], f2 = row[j + 2];
      const T vm2 = vrow[j - 2], vm1 = vrow[j - 1], v0 = vrow[j], v1 = vrow[j + 1],
              v2 = vrow[j + 2];
      // y direction (r axis): rows i-2 .. i+2 of column j through the mirror
      const T gm2 = mir(src, i - 2, j, nz, par), gm1 = mir(src, i - 1, j, nz, par);
      const T g1 = src[c + nz], g2 = src[c + 2LL * nz];
      const T wm2 = mir(ur, i - 2, j, nz, T(-1)), wm1 = mir(ur, i - 1, j, nz, T(-1));
      const T w0 = ur[c], w1 = ur[c + nz], w2 = ur[c + 2LL * nz];
      if (CONS) {
        const T xf = face_cons(fm1, f0, f1, f2, vm1, v0, v1, v2);
        const T xb = face_cons(fm2, fm1, f0, f1, vm2, vm1, v0, v1);
        const T yf = face_cons(gm1, f0, g1, g2, wm1, w0, w1, w2);
        const T yb = face_cons(gm2, gm1, f0, g1, wm2, wm1, w0, w1);
        flux = rn_add(flux, rn_mul(a, xf));
        flux = rn_sub(flux, rn_mul(a, xb));
        flux = rn_add(flux, rn_mul(a, yf));
        flux = rn_sub(flux, rn_mul(a, yb));
      } else {
        const T xf = face_noncons(fm1, f0, f1, f2, v0, v1);
        const T xb = face_noncons(fm2, fm1, f0, f1, vm1, v0);
        const T yf = face_noncons(gm1, f0, g1, g2, w0, w1);
        const T yb = face_noncons(gm2, gm1, f0, g1, wm1, w0);
        flux = rn_add(flux, rn_mul(rn_mul(a, xf), v0));
        flux = rn_sub(flux, rn_mul(rn_mul(a, xb), v0));
        flux = rn_add(flux, rn_mul(rn_mul(a, yf), w0));
        flux = rn_sub(flux, rn_mul(rn_mul(a, yb), w0));
      }
    }
    dst[c] = rn_add(src[c], flux);
  }
}

template <typename T, int NF, bool CONS>
int eno3_launch(T* f0, T* f1, T par0, T par1, const T* uz, const T* ur, T* scratch, int nr,
                int nz, T dt_by_dx, cudaStream_t s, const char* what,
                const double* dt_dev = nullptr, T dx = T(0)) {
  if (nr < 3 || nz < 5) {
    axi::set_error("%s: grid %d x %d too small for ENO3 (needs nr >= 3, nz >= 5)", what, nr, nz);
    return AXI_ERR_INVALID;
  }
  AXI_TRY(axi::check_ptrs(what, {f0, uz, ur, scratch},
                          {NF == 2 ? "eta1" : "vorticity", "u_z", "u_r", "scratch"}));
  if (NF == 2) AXI_TRY(axi::check_ptr(what, f1, "eta2"));
  const size_t bytes = (size_t)nr * nz * sizeof(T);
  if (cudaMemcpyAsync(scratch, f0, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return axi::launch_status(what);
  T* s1 = nullptr;
  if (NF == 2) {
    s1 = scratch + (size_t)nr * nz;
    if (cudaMemcpyAsync(s1, f1, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return axi::launch_status(what);
  }
  dim3 grid(axi::ceil_div(nz, BX), axi::ceil_div(nr, BY));
  eno3_step_kernel<T, NF, CONS><<<grid, dim3(BX, BY), 0, s>>>(f0, f1, scratch, s1, par0, par1,
                                                              uz, ur, nr, nz, -dt_by_dx,
                                                              dt_dev, dx);
  return axi::launch_status(what);
}

}  // namespace

#define AXI_DEFINE_ENO3(SUF, T)                                                                \
  extern "C" int axi_advect_vorticity_eno3_##SUF(T* vort, const T* u_z, const T* u_r,          \
                                                 T* scratch, int nr, int nz, T dt_by_dx,       \
                                                 void* stream) {                               \
    axi::clear_error();                                                                        \
    return eno3_launch<T, 1, true>(vort, nullptr, T(-1), T(0), u_z, u_r, scratch, nr, nz,      \
                                   dt_by_dx, axi::as_stream(stream), "advect_vorticity_eno3"); \
  }                                                                                            \
  extern "C" int axi_advect_vorticity_eno3_periodic_##SUF(T* vort, T* u_z, T* u_r, T* scratch, \
                                                          int nr, int nz, T dt_by_dx,          \
                                                          int ghost, void* stream) {           \
    axi::clear_error();                                                                        \
    AXI_TRY(axi_periodic_ghost_comm_##SUF(u_z, nr, nz, ghost, stream));                        \
    AXI_TRY(axi_periodic_ghost_comm_##SUF(u_r, nr, nz, ghost, stream));                        \
    AXI_TRY(axi_periodic_ghost_comm_##SUF(vort, nr, nz, ghost, stream));                       \
    return eno3_launch<T, 1, true>(vort, nullptr, T(-1), T(0), u_z, u_r, scratch, nr, nz,      \
                                   dt_by_dx, axi::as_stream(stream),                           \
                                   "advect_vorticity_eno3_periodic");                          \
  }                                                                                            \
  extern "C" int axi_advect_refmap_eno3_##SUF(T* eta1, T* eta2, const T* u_z, const T* u_r,    \
                                              T* scratch2, int nr, int nz, T dt_by_dx,         \
                                              void* stream) {                                  \
    axi::clear_error();                                                                        \
    return eno3_launch<T, 2, false>(eta1, eta2, T(1), T(-1), u_z, u_r, scratch2, nr, nz,       \
                                    dt_by_dx, axi::as_stream(stream), "advect_refmap_eno3");   \
  }                                                                                            \
  extern "C" int axi_advect_refmap_eno3_periodic_##SUF(T* eta1, T* eta2, T* u_z, T* u_r,       \
                                                       T* scratch2, int nr, int nz,            \
                                                       T dt_by_dx, int ghost, T z_max, T dx,   \
                                                       void* stream) {                         \
    axi::clear_error();                                                                        \
    AXI_TRY(axi_periodic_ghost_comm_##SUF(u_z, nr, nz, ghost, stream));                        \
    AXI_TRY(axi_periodic_ghost_comm_##SUF(u_r, nr, nz, ghost, stream));                        \
    AXI_TRY(axi_periodic_ghost_comm_eta_##SUF(eta1, nr, nz, ghost, z_max, dx, stream));        \
    AXI_TRY(axi_periodic_ghost_comm_##SUF(eta2, nr, nz, ghost, stream));                       \
    return eno3_launch<T, 2, false>(eta1, eta2, T(1), T(-1), u_z, u_r, scratch2, nr, nz,       \
                                    dt_by_dx, axi::as_stream(stream),                          \
                                    "advect_refmap_eno3_periodic");                            \
  }

AXI_DEFINE_ENO3(f64, double)
AXI_DEFINE_ENO3(f32, float)

// The soft-sphere loop's two advections with the time step read on the device
// (state[AXI_SOFT_DT]): eta (non-conservative, eta1 even and eta2 odd about the
// axis, elasto_kernels/advect_refmap_via_eno3.py:8-44) or omega (conservative,
// odd), the arithmetic of the host-dt entries above.
extern "C" int axi_soft_advect_eno3_f64(double* f0, double* f1, int refmap, const double* u_z,
                                        const double* u_r, double* scratch, int nr, int nz,
                                        double dx, const double* state, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptrs("soft_advect_eno3", {f0, u_z, u_r, scratch, state},
                          {refmap ? "eta1" : "omega", "u_z", "u_r", "scratch", "state"}));
  if (refmap) {
    AXI_TRY(axi::check_ptr("soft_advect_eno3", f1, "eta2"));
    return eno3_launch<double, 2, false>(f0, f1, 1.0, -1.0, u_z, u_r, scratch, nr, nz, 0.0,
                                         axi::as_stream(stream), "soft_advect_eno3",
                                         state + AXI_SOFT_DT, dx);
  }
  return eno3_launch<double, 1, true>(f0, nullptr, -1.0, 0.0, u_z, u_r, scratch, nr, nz, 0.0,
                                      axi::as_stream(stream), "soft_advect_eno3",
                                      state + AXI_SOFT_DT, dx);
}
