// Device-resident pieces of the soft-sphere streaming loop
// (examples/SoftSphereStreaming/soft_sphere_streaming.py:129-272), FP64.
//
// The drop-in kernels of the loop take the time step and the simulated time
// as host scalars, so a host loop reads max |u| back every step to form dt.
// Here dt and t live in a small state block on the device (AXI_SOFT_*
// words): one kernel reduces max(|u_z| + |u_r|) and forms dt, the dt- and
// t-dependent kernels read it there, and the step runs without a host round
// trip (and can be captured in a CUDA graph). Each kernel keeps the operation
// order of the drop-in kernel (or torch expression) it replaces, with the *_rn
// intrinsics, so results match the host-dt loop; only sin / cos of omega t
// are evaluated on the device instead of the host.
#include <algorithm>

#include "axi_common.cuh"

namespace {

constexpr int NT = 256;

inline int blocks_for(long long n) { return axi::ceil_div(n, NT); }

// dt = min(cfl dx / sqrt(G / rho_f), cfl dx / (max(|u_z| + |u_r|) + eps),
//          0.9 dx^2 / 4 / nu)   (soft_sphere_streaming.py:168-172; the plotting
// clip of :173-176 is not part of the loop here)
// Block maxima go to the state word AXI_SOFT_UMAX as ordered bit patterns
// (non-negative doubles order like their bits); the last block to arrive
// forms dt and clears the maximum and the arrival count for the next step.
__global__ void __launch_bounds__(NT) dt_kernel(const double* __restrict__ uz,
                                                const double* __restrict__ ur, long long n,
                                                double* state, double dt_elastic, double cfl_dx,
                                                double dt_diffusive, double eps) {
  __shared__ unsigned long long red[NT / 32];
  __shared__ bool last;
  unsigned long long m = 0;
  for (long long k = (long long)blockIdx.x * NT + threadIdx.x; k < n;
       k += (long long)gridDim.x * NT) {
    const double v = __dadd_rn(fabs(uz[k]), fabs(ur[k]));
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    m = b > m ? b : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_down_sync(0xffffffffu, m, o);
    m = x > m ? x : m;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  unsigned long long* words = reinterpret_cast<unsigned long long*>(state);
  if (threadIdx.x == 0) {
    unsigned long long bm = 0;
    for (int q = 0; q < NT / 32; ++q) bm = red[q] > bm ? red[q] : bm;
    atomicMax(&words[AXI_SOFT_UMAX], bm);
    __threadfence();
    last = atomicAdd(&words[AXI_SOFT_COUNT], 1ull) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  const double umax = __longlong_as_double(
      (long long)atomicAdd(&words[AXI_SOFT_UMAX], 0ull));
  // Python's min(a, b, c): the first of the smallest
  double dt = dt_elastic;
  const double cfl = __ddiv_rn(cfl_dx, __dadd_rn(umax, eps));
  if (cfl < dt) dt = cfl;
  if (dt_diffusive < dt) dt = dt_diffusive;
  if (!(umax == umax))
    atomicOr(&words[AXI_SOFT_STATUS], 1ull << AXI_ERR_NONFINITE);
  state[AXI_SOFT_DT] = dt;
  words[AXI_SOFT_UMAX] = 0ull;
  words[AXI_SOFT_COUNT] = 0ull;
}

// Level set pinned to the advected reference map inside the band
// phi > -3 dx (soft_sphere_streaming.py:191-193):
// phi = where(phi > band, -sqrt((eta1 - z_cm)^2 + eta2^2) + r_ball, phi)
__global__ void __launch_bounds__(NT) pin_kernel(double* __restrict__ phi,
                                                 const double* __restrict__ e1,
                                                 const double* __restrict__ e2, long long n,
                                                 double z_cm, double r_ball, double band) {
  const long long k = (long long)blockIdx.x * NT + threadIdx.x;
  if (k >= n) return;
  const double p = phi[k];
  if (p > band) {
    const double d = __dsub_rn(e1[k], z_cm);
    const double s = __dadd_rn(__dmul_rn(d, d), __dmul_rn(e2[k], e2[k]));
    phi[k] = __dadd_rn(-__dsqrt_rn(s), r_ball);
  }
}

// smooth_Heaviside (kernels/smooth_Heaviside.py:10-14, the drop-in kernel's
// order) of phi into H, and inside = H > 0.5
__device__ __forceinline__ double heaviside(double h_old, double p, double w) {
  double h = __dmul_rn(0.0, h_old);
  h = __dadd_rn(h, (p >= w) ? 1.0 : 0.0);
  const double a = __dadd_rn(1.0, __ddiv_rn(p, w));
  const double s = __ddiv_rn(sin(__ddiv_rn(__dmul_rn(Pi<double>::v, p), w)), Pi<double>::v);
  const double m05 = (fabs(p) < w) ? 0.5 : 0.0;
  return __dadd_rn(h, __dmul_rn(m05, __dadd_rn(a, s)));
}

__global__ void __launch_bounds__(NT) mask_kernel(double* __restrict__ H,
                                                  uint8_t* __restrict__ inside,
                                                  const double* __restrict__ phi, long long n,
                                                  double w) {
  const long long k = (long long)blockIdx.x * NT + threadIdx.x;
  if (k >= n) return;
  const double h = heaviside(H[k], phi[k], w);
  H[k] = h;
  inside[k] = h > 0.5 ? 1 : 0;
}

// sigma *= chi (soft_sphere_streaming.py:236-238)
__global__ void __launch_bounds__(NT) stress_mask_kernel(double* __restrict__ s11,
                                                         double* __restrict__ s12,
                                                         double* __restrict__ s22,
                                                         const double* __restrict__ chi,
                                                         long long n) {
  const long long k = (long long)blockIdx.x * NT + threadIdx.x;
  if (k >= n) return;
  const double c = chi[k];
  s11[k] = __dmul_rn(s11[k], c);
  s12[k] = __dmul_rn(s12[k], c);
  s22[k] = __dmul_rn(s22[k], c);
}

// Tether mask at the oscillating centre z_cm + e r_ball sin(omega t)
// (soft_sphere_streaming.py:243-245): level set
// -sqrt((Z - z_t)^2 + R^2) + zeta r_ball, smoothed Heaviside.
__global__ void __launch_bounds__(NT) tether_kernel(double* __restrict__ H,
                                                    const double* __restrict__ Z,
                                                    const double* __restrict__ R, long long n,
                                                    const double* __restrict__ state, double z_cm,
                                                    double e_r, double omega, double zeta_r,
                                                    double w) {
  const long long k = (long long)blockIdx.x * NT + threadIdx.x;
  if (k >= n) return;
  const double zt = __dadd_rn(z_cm, __dmul_rn(e_r, sin(__dmul_rn(omega, state[AXI_SOFT_T]))));
  const double d = __dsub_rn(Z[k], zt);
  const double r = R[k];
  const double p = __dadd_rn(-__dsqrt_rn(__dadd_rn(__dmul_rn(d, d), __dmul_rn(r, r))), zeta_r);
  H[k] = heaviside(H[k], p, w);
}

// Brinkman penalisation towards (U0 cos(omega t), 0)
// (soft_sphere_streaming.py:248-260, kernels/brinkmann_penalize.py:11-16):
// u <- (u + lam dt chi U) / (1 + lam dt chi); d = u_pen - u into d_z, d_r.
__global__ void __launch_bounds__(NT) brinkman_kernel(double* __restrict__ uz,
                                                      double* __restrict__ ur,
                                                      const double* __restrict__ chi,
                                                      double* __restrict__ dz,
                                                      double* __restrict__ dr, long long n,
                                                      const double* __restrict__ state,
                                                      double lam, double U0, double omega) {
  const long long k = (long long)blockIdx.x * NT + threadIdx.x;
  if (k >= n) return;
  const double Uz = __dmul_rn(U0, cos(__dmul_rn(omega, state[AXI_SOFT_T])));
  const double ldt = __dmul_rn(lam, state[AXI_SOFT_DT]);
  const double lc = __dmul_rn(ldt, chi[k]);
  const double den = __dadd_rn(1.0, lc);
  const double vz = uz[k], vr = ur[k];
  const double pz = __ddiv_rn(__dadd_rn(vz, __dmul_rn(lc, Uz)), den);
  const double pr = __ddiv_rn(__dadd_rn(vr, __dmul_rn(lc, 0.0)), den);
  dz[k] = __dsub_rn(pz, vz);
  dr[k] = __dsub_rn(pr, vr);
  uz[k] = pz;
  ur[k] = pr;
}

// omega += curl(u_pen - u) on the interior (kernels/compute_vorticity_from_velocity.py:11-13,
// then omega += penal; soft_sphere_streaming.py:261-264)
__global__ void __launch_bounds__(NT) penal_curl_kernel(double* __restrict__ w,
                                                        const double* __restrict__ dz,
                                                        const double* __restrict__ dr, int nr,
                                                        int nz, double dx) {
  const long long k = (long long)blockIdx.x * NT + threadIdx.x;
  if (k >= (long long)nr * nz) return;
  const int i = (int)(k / nz), j = (int)(k - (long long)i * nz);
  if (i < 1 || j < 1 || i >= nr - 1 || j >= nz - 1) return;
  const double two_dx = __dmul_rn(2.0, dx);
  const double a = __ddiv_rn(__dsub_rn(dr[k + 1], dr[k - 1]), two_dx);
  const double b = __ddiv_rn(__dsub_rn(dz[k + nz], dz[k - nz]), two_dx);
  w[k] = __dadd_rn(w[k], __dsub_rn(a, b));
}

// t += dt, steps += 1 (soft_sphere_streaming.py:270-272)
__global__ void advance_kernel(double* state) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  state[AXI_SOFT_T] = __dadd_rn(state[AXI_SOFT_T], state[AXI_SOFT_DT]);
  state[AXI_SOFT_STEPS] += 1.0;
}

int check_n(const char* what, long long n) {
  if (n <= 0) {
    axi::set_error("%s: empty field", what);
    return AXI_ERR_INVALID;
  }
  return AXI_OK;
}

}  // namespace

extern "C" int axi_soft_dt_f64(const double* u_z, const double* u_r, int64_t n, double* state,
                               double dt_elastic, double cfl_dx, double dt_diffusive, double eps,
                               void* stream) {
  axi::clear_error();
  AXI_TRY(check_n("soft_dt", n));
  AXI_TRY(axi::check_ptrs("soft_dt", {u_z, u_r, state}, {"u_z", "u_r", "state"}));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = std::min<long long>(blocks_for(n), 4LL * (sms > 0 ? sms : 1));
  dt_kernel<<<blocks, NT, 0, axi::as_stream(stream)>>>(u_z, u_r, n, state, dt_elastic, cfl_dx,
                                                       dt_diffusive, eps);
  return axi::launch_status("soft_dt");
}

extern "C" int axi_soft_pin_level_set_f64(double* ball_phi, const double* eta1,
                                          const double* eta2, int64_t n, double z_cm,
                                          double r_ball, double band, void* stream) {
  axi::clear_error();
  AXI_TRY(check_n("soft_pin_level_set", n));
  AXI_TRY(axi::check_ptrs("soft_pin_level_set", {ball_phi, eta1, eta2},
                          {"ball_phi", "eta1", "eta2"}));
  pin_kernel<<<blocks_for(n), NT, 0, axi::as_stream(stream)>>>(ball_phi, eta1, eta2, n, z_cm,
                                                              r_ball, band);
  return axi::launch_status("soft_pin_level_set");
}

extern "C" int axi_soft_mask_f64(double* chi, uint8_t* inside, const double* phi, int64_t n,
                                 double blend_w, void* stream) {
  axi::clear_error();
  AXI_TRY(check_n("soft_mask", n));
  AXI_TRY(axi::check_ptrs("soft_mask", {chi, inside, phi}, {"chi", "inside", "phi"}));
  mask_kernel<<<blocks_for(n), NT, 0, axi::as_stream(stream)>>>(chi, inside, phi, n, blend_w);
  return axi::launch_status("soft_mask");
}

extern "C" int axi_soft_stress_mask_f64(double* s11, double* s12, double* s22, const double* chi,
                                        int64_t n, void* stream) {
  axi::clear_error();
  AXI_TRY(check_n("soft_stress_mask", n));
  AXI_TRY(axi::check_ptrs("soft_stress_mask", {s11, s12, s22, chi}, {"s11", "s12", "s22", "chi"}));
  stress_mask_kernel<<<blocks_for(n), NT, 0, axi::as_stream(stream)>>>(s11, s12, s22, chi, n);
  return axi::launch_status("soft_stress_mask");
}

extern "C" int axi_soft_tether_f64(double* tether_chi, const double* Z, const double* R,
                                   int64_t n, const double* state, double z_cm, double e_r_ball,
                                   double omega, double zeta_r_ball, double blend_w,
                                   void* stream) {
  axi::clear_error();
  AXI_TRY(check_n("soft_tether", n));
  AXI_TRY(axi::check_ptrs("soft_tether", {tether_chi, Z, R, state},
                          {"tether_chi", "Z", "R", "state"}));
  tether_kernel<<<blocks_for(n), NT, 0, axi::as_stream(stream)>>>(
      tether_chi, Z, R, n, state, z_cm, e_r_ball, omega, zeta_r_ball, blend_w);
  return axi::launch_status("soft_tether");
}

extern "C" int axi_soft_penalise_f64(double* omega, double* u_z, double* u_r,
                                     const double* tether_chi, double* d_z, double* d_r, int nr,
                                     int nz, double dx, double lam, double U0, double omega_f,
                                     const double* state, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_grid("soft_penalise", nr, nz));
  AXI_TRY(axi::check_ptrs("soft_penalise", {omega, u_z, u_r, tether_chi, d_z, d_r, state},
                          {"omega", "u_z", "u_r", "tether_chi", "d_z", "d_r", "state"}));
  const long long n = (long long)nr * nz;
  cudaStream_t s = axi::as_stream(stream);
  brinkman_kernel<<<blocks_for(n), NT, 0, s>>>(u_z, u_r, tether_chi, d_z, d_r, n, state, lam, U0,
                                               omega_f);
  penal_curl_kernel<<<blocks_for(n), NT, 0, s>>>(omega, d_z, d_r, nr, nz, dx);
  return axi::launch_status("soft_penalise");
}

extern "C" int axi_soft_advance_f64(double* state, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("soft_advance", state, "state"));
  advance_kernel<<<1, 32, 0, axi::as_stream(stream)>>>(state);
  return axi::launch_status("soft_advance");
}
