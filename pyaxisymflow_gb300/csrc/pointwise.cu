// Pointwise and nearest-neighbour grid kernels of the per-timestep hot path.
//
// One thread per cell, z (the contiguous axis) on threadIdx.x so every warp
// reads and writes 32 consecutive doubles. Where the reference kernel has no
// transcendental function the arithmetic is issued with the *_rn intrinsics
// in the reference's own evaluation order, so results are bit-identical to the
// numpy evaluation of the reference (no FMA contraction).
#include "axi_common.cuh"

namespace {

constexpr int BX = 32;
constexpr int BY = 8;

inline dim3 grid2d(int nr, int nz) { return dim3(axi::ceil_div(nz, BX), axi::ceil_div(nr, BY)); }

// kernels/compute_velocity_from_psi.py:9-17
template <typename T>
__global__ void velocity_from_psi_kernel(T* __restrict__ u_z, T* __restrict__ u_r,
                                         const T* __restrict__ psi, const T* __restrict__ R,
                                         int nr, int nz, T dx) {
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  if (i >= nr || j >= nz) return;
  const long long c = (long long)i * nz + j;
  const T two_dx = rn_mul(T(2), dx);
  const T r = R[c];
  T dz;
  if (i == 0) {
    // (-psi[2] + 4 psi[1] - 3 psi[0]) / (2 dx) / R[0]
    T a = rn_add(-psi[2LL * nz + j], rn_mul(T(4), psi[(long long)nz + j]));
    dz = rn_sub(a, rn_mul(T(3), psi[j]));
  } else if (i == nr - 1) {
    // (psi[-3] - 4 psi[-2] + 3 psi[-1])
    T a = rn_sub(psi[c - 2LL * nz], rn_mul(T(4), psi[c - nz]));
    dz = rn_add(a, rn_mul(T(3), psi[c]));
  } else {
    dz = rn_sub(psi[c + nz], psi[c - nz]);
  }
  u_z[c] = rn_div(rn_div(dz, two_dx), r);
  T dr;
  if (j == 0) {
    T a = rn_add(-psi[c + 2], rn_mul(T(4), psi[c + 1]));
    dr = rn_sub(a, rn_mul(T(3), psi[c]));
  } else if (j == nz - 1) {
    T a = rn_sub(psi[c - 2], rn_mul(T(4), psi[c - 1]));
    dr = rn_add(a, rn_mul(T(3), psi[c]));
  } else {
    dr = rn_sub(psi[c + 1], psi[c - 1]);
  }
  u_r[c] = rn_div(rn_div(-dr, two_dx), r);
}

// kernels/periodic_boundary_ghost_comm.py:9-13 (shift == 0) and :23-31 (eta):
// field[:, :g] = field[:, -2g:-g] - shift; field[:, -g:] = field[:, g:2g] + shift,
// shift = z_max - 2 g dx (applied in the reference's order: a - z_max + 2 g dx).
template <typename T>
__global__ void ghost_comm_kernel(T* __restrict__ f, int nr, int nz, int g, bool eta, T z_max,
                                  T two_g_dx) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;  // 0 .. 2g-1
  const int i = blockIdx.y;
  if (k >= 2 * g || i >= nr) return;
  T* row = f + (long long)i * nz;
  if (k < g) {
    T v = row[nz - 2 * g + k];
    row[k] = eta ? rn_add(rn_sub(v, z_max), two_g_dx) : v;
  } else {
    const int kk = k - g;
    T v = row[g + kk];
    row[nz - g + kk] = eta ? rn_sub(rn_add(v, z_max), two_g_dx) : v;
  }
}

// kernels/compute_vorticity_from_velocity.py:11-13 on [1:-1, 1:-1]
template <typename T>
__global__ void vorticity_from_velocity_kernel(T* __restrict__ vort, const T* __restrict__ u_z,
                                               const T* __restrict__ u_r, int nr, int nz, T dx) {
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  if (i < 1 || j < 1 || i >= nr - 1 || j >= nz - 1) return;
  const long long c = (long long)i * nz + j;
  const T two_dx = rn_mul(T(2), dx);
  T a = rn_div(rn_sub(u_r[c + 1], u_r[c - 1]), two_dx);
  T b = rn_div(rn_sub(u_z[c + nz], u_z[c - nz]), two_dx);
  vort[c] = rn_sub(a, b);
}

// kernels/brinkmann_penalize.py:11-16
template <typename T>
__global__ void brinkman_kernel(T lam, T dt, const T* __restrict__ chi, T U_z, T U_r,
                                const T* __restrict__ gz, const T* __restrict__ gr,
                                T* __restrict__ pz, T* __restrict__ pr, long long n) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const T ldt = rn_mul(lam, dt);
  const T lc = rn_mul(ldt, chi[k]);
  const T denom = rn_add(T(1), lc);
  const T vz = gz[k], vr = gr[k];
  pz[k] = rn_div(rn_add(vz, rn_mul(lc, U_z)), denom);
  pr[k] = rn_div(rn_add(vr, rn_mul(lc, U_r)), denom);
}

// kernels/smooth_Heaviside.py:10-14
template <typename T>
__global__ void heaviside_kernel(T* __restrict__ H, const T* __restrict__ phi, T w, long long n) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const T p = phi[k];
  T h = rn_mul(T(0), H[k]);
  h = rn_add(h, (p >= w) ? T(1) : T(0));
  // (|phi| < w) * 0.5 * (1 + phi / w + sin(pi * phi / w) / pi), left to right
  const T a = rn_add(T(1), rn_div(p, w));
  const T s = rn_div(dev_sin(rn_div(rn_mul(Pi<T>::v, p), w)), Pi<T>::v);
  const T m05 = (fabs(p) < w) ? T(0.5) : T(0);
  h = rn_add(h, rn_mul(m05, rn_add(a, s)));
  H[k] = h;
}

// kernels/kill_boundary_vorticity_sine.py:9-14: both z strips of width w. Each
// thread owns one row; the source columns are read before any write.
template <typename T>
__global__ void kill_z_kernel(T* __restrict__ vort, const T* __restrict__ Z, int nr, int nz,
                              int w, T dx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nr) return;
  T* row = vort + (long long)i * nz;
  const T* zr = Z + (long long)i * nz;
  const T half_dx = rn_mul(T(0.5), dx);
  const T left = row[w - 1];
  // The right strip is assigned after the left one (numpy statement order), so
  // its source column -w sees the left update when the strips overlap.
  T newleft[8];
  for (int k = 0; k < w && k < 8; ++k) {
    T arg = rn_div(rn_div(rn_div(rn_mul(Pi<T>::v, rn_sub(zr[k], half_dx)), T(2)), T(w - 1)), dx);
    newleft[k] = rn_mul(dev_sin(arg), left);
  }
  for (int k = 0; k < w && k < 8; ++k) row[k] = newleft[k];
  const T right = row[nz - w];
  T newright[8];
  for (int k = 0; k < w && k < 8; ++k) {
    const int j = nz - w + k;
    T arg = rn_div(rn_div(rn_div(rn_mul(Pi<T>::v, rn_sub(rn_sub(T(1), zr[j]), half_dx)), T(2)),
                          T(w - 1)), dx);
    newright[k] = rn_mul(dev_sin(arg), right);
  }
  for (int k = 0; k < w && k < 8; ++k) row[nz - w + k] = newright[k];
}

// kernels/kill_boundary_vorticity_sine.py:23-27: outer-r strip, then row 0 = 0.
// Each thread owns one column.
template <typename T>
__global__ void kill_r_kernel(T* __restrict__ vort, const T* __restrict__ R, int nr, int nz,
                              int w, T dx) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nz) return;
  const T half_dx = rn_mul(T(0.5), dx);
  const T src = vort[(long long)(nr - w) * nz + j];
  for (int k = 0; k < w; ++k) {
    const long long c = (long long)(nr - w + k) * nz + j;
    T arg = rn_div(rn_div(rn_div(rn_mul(Pi<T>::v, rn_sub(rn_sub(T(1), R[c]), half_dx)), T(2)),
                          T(w - 1)), dx);
    vort[c] = rn_mul(dev_sin(arg), src);
  }
  vort[j] = T(0);
}

// kernels/diffusion_RK2.py:15-25: the bracketed operator at interior cell c.
template <typename T>
__device__ __forceinline__ T rk2_operator(const T* __restrict__ w, const T* __restrict__ R,
                                          long long c, int nz, T dx2, T two_dx) {
  const T n = w[c + nz], s = w[c - nz], e = w[c + 1], wst = w[c - 1], ctr = w[c];
  const T r = R[c];
  T lap = rn_add(rn_add(rn_add(n, s), e), wst);
  lap = rn_div(rn_sub(lap, rn_mul(T(4), ctr)), dx2);
  const T adv = rn_div(rn_div(rn_sub(n, s), two_dx), r);
  const T inv_r2 = rn_div(T(1), rn_mul(r, r));
  return rn_sub(rn_add(lap, adv), rn_mul(ctr, inv_r2));
}

// diffusion_RK2.py:9-26: temp = vort; temp[1:-1,1:-1] += 0.5 nu dt L(vort)
template <typename T>
__global__ void rk2_stage1_kernel(const T* __restrict__ w, T* __restrict__ tmp,
                                  const T* __restrict__ R, int nr, int nz, T coef, T dx2,
                                  T two_dx, const double* __restrict__ dt_dev = nullptr) {
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  if (i >= nr || j >= nz) return;
  // device-resident time step: coef holds the factor of dt ((0.5 nu) or nu)
  if (dt_dev) coef = rn_mul(coef, static_cast<T>(dt_dev[0]));
  const long long c = (long long)i * nz + j;
  T v = w[c];
  if (i > 0 && j > 0 && i < nr - 1 && j < nz - 1)
    v = rn_add(v, rn_mul(coef, rk2_operator(w, R, c, nz, dx2, two_dx)));
  tmp[c] = v;
}

// diffusion_RK2.py:27-44: vort[1:-1,1:-1] += nu dt L(temp)
template <typename T>
__global__ void rk2_stage2_kernel(T* __restrict__ w, const T* __restrict__ tmp,
                                  const T* __restrict__ R, int nr, int nz, T coef, T dx2,
                                  T two_dx, const double* __restrict__ dt_dev = nullptr) {
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  if (i < 1 || j < 1 || i >= nr - 1 || j >= nz - 1) return;
  if (dt_dev) coef = rn_mul(coef, static_cast<T>(dt_dev[0]));
  const long long c = (long long)i * nz + j;
  w[c] = rn_add(w[c], rn_mul(coef, rk2_operator(tmp, R, c, nz, dx2, two_dx)));
}

// elasto_kernels/solid_sigma.py:18-29: gradients where the reference writes
// them, then the stress from whatever the gradient arrays hold.
template <typename T>
__global__ void solid_sigma_kernel(T* __restrict__ s11, T* __restrict__ s12, T* __restrict__ s22,
                                   T G, T dx, const T* __restrict__ e1, const T* __restrict__ e2,
                                   T* __restrict__ e1z, T* __restrict__ e1r, T* __restrict__ e2z,
                                   T* __restrict__ e2r, int nr, int nz) {
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  if (i >= nr || j >= nz) return;
  const long long c = (long long)i * nz + j;
  const T two_dx = rn_mul(T(2), dx);
  T g1z = e1z[c], g2z = e2z[c], g1r = e1r[c], g2r = e2r[c];
  if (j > 0 && j < nz - 1) {
    g1z = rn_div(rn_sub(e1[c + 1], e1[c - 1]), two_dx);
    g2z = rn_div(rn_sub(e2[c + 1], e2[c - 1]), two_dx);
    e1z[c] = g1z;
    e2z[c] = g2z;
  }
  if (i == 0) {
    g1r = rn_div(rn_sub(rn_add(-e1[2LL * nz + j], rn_mul(T(4), e1[(long long)nz + j])),
                        rn_mul(T(3), e1[j])), two_dx);
    g2r = rn_div(rn_sub(rn_add(-e2[2LL * nz + j], rn_mul(T(4), e2[(long long)nz + j])),
                        rn_mul(T(3), e2[j])), two_dx);
    e1r[c] = g1r;
    e2r[c] = g2r;
  } else if (i < nr - 1 && j > 0 && j < nz - 1) {
    g1r = rn_div(rn_sub(e1[c + nz], e1[c - nz]), two_dx);
    g2r = rn_div(rn_sub(e2[c + nz], e2[c - nz]), two_dx);
    e1r[c] = g1r;
    e2r[c] = g2r;
  }
  const T v12 = rn_mul(-G, rn_add(rn_mul(g1z, g1r), rn_mul(g2z, g2r)));
  T t = rn_add(rn_mul(g1r, g1r), rn_mul(g2r, g2r));
  t = rn_sub(rn_sub(t, rn_mul(g1z, g1z)), rn_mul(g2z, g2z));
  const T v11 = rn_mul(rn_mul(T(0.5), G), t);
  s12[c] = v12;
  s11[c] = v11;
  s22[c] = -v11;
}

// elasto_kernels/div_tau.py:8-28: tau on [1:-1, 1:-1] and row 0 [0, 1:-1].
template <typename T>
__global__ void div_tau_kernel(T* __restrict__ tz, T* __restrict__ tr, const T* __restrict__ t11,
                               const T* __restrict__ t12, const T* __restrict__ t22,
                               const T* __restrict__ R, int nr, int nz, T dx) {
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  if (i >= nr - 1 || j < 1 || j >= nz - 1) return;
  const long long c = (long long)i * nz + j;
  const T two_dx = rn_mul(T(2), dx);
  const T r = R[c];
  if (i == 0) {
    T a = rn_sub(rn_sub(t11[c + 1], t11[c - 1]), t12[c + 2LL * nz]);
    a = rn_sub(rn_add(a, rn_mul(T(4), t12[c + nz])), rn_mul(T(3), t12[c]));
    tz[c] = rn_add(rn_div(a, two_dx), rn_div(t12[c], r));
    T b = rn_sub(rn_sub(t12[c + 1], t12[c - 1]), t22[c + 2LL * nz]);
    b = rn_sub(rn_add(b, rn_mul(T(4), t22[c + nz])), rn_mul(T(3), t22[c]));
    tr[c] = rn_add(rn_div(b, two_dx), rn_div(t22[c], r));
  } else {
    T a = rn_add(rn_sub(t11[c + 1], t11[c - 1]), t12[c + nz]);
    a = rn_sub(a, t12[c - nz]);
    tz[c] = rn_add(rn_div(a, two_dx), rn_div(t12[c], r));
    T b = rn_add(rn_sub(t12[c + 1], t12[c - 1]), t22[c + nz]);
    b = rn_sub(b, t22[c - nz]);
    tr[c] = rn_add(rn_div(b, two_dx), rn_div(t22[c], r));
  }
}

// elasto_kernels/div_tau.py:30-34: vort[1:-1,1:-1] += dt (dtau_r/dz - dtau_z/dr) / (2 dx)
template <typename T>
__global__ void curl_tau_kernel(T* __restrict__ w, const T* __restrict__ tz,
                                const T* __restrict__ tr, int nr, int nz, T dt, T dx,
                                const double* __restrict__ dt_dev = nullptr) {
  const int j = blockIdx.x * BX + threadIdx.x;
  const int i = blockIdx.y * BY + threadIdx.y;
  if (i < 1 || j < 1 || i >= nr - 1 || j >= nz - 1) return;
  if (dt_dev) dt = static_cast<T>(dt_dev[0]);
  const long long c = (long long)i * nz + j;
  T a = rn_sub(rn_sub(tr[c + 1], tr[c - 1]), tz[c + nz]);
  a = rn_add(a, tz[c - nz]);
  w[c] = rn_add(w[c], rn_div(rn_mul(dt, a), rn_mul(T(2), dx)));
}

template <typename T>
int ghost_comm(T* f, int nr, int nz, int g, bool eta, T z_max, T dx, cudaStream_t s) {
  if (g <= 0 || nz < 4 * g || nr < 1 || nr > 65535) {
    axi::set_error("periodic_ghost_comm: invalid ghost size %d for nz = %d", g, nz);
    return AXI_ERR_INVALID;
  }
  AXI_TRY(axi::check_ptr("periodic_ghost_comm", f, "field"));
  const int threads = 2 * g <= 256 ? 2 * g : 256;
  dim3 grid(axi::ceil_div(2 * g, threads), nr);
  ghost_comm_kernel<T><<<grid, threads, 0, s>>>(f, nr, nz, g, eta, z_max,
                                                 rn_host_mul(T(2 * g), dx));
  return axi::launch_status("periodic_ghost_comm");
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

#define AXI_DEFINE_VELOCITY(SUF, T)                                                           \
  extern "C" int axi_velocity_from_psi_unb_##SUF(T* u_z, T* u_r, const T* psi, const T* R,    \
                                                 int nr, int nz, T dx, void* stream) {        \
    axi::clear_error();                                                                       \
    AXI_TRY(axi::check_grid("velocity_from_psi", nr, nz));                                    \
    AXI_TRY(axi::check_ptrs("velocity_from_psi", {u_z, u_r, psi, R},                           \
                            {"u_z", "u_r", "psi", "R"}));                                      \
    velocity_from_psi_kernel<T><<<grid2d(nr, nz), dim3(BX, BY), 0, axi::as_stream(stream)>>>( \
        u_z, u_r, psi, R, nr, nz, dx);                                                        \
    return axi::launch_status("velocity_from_psi");                                           \
  }                                                                                           \
  extern "C" int axi_velocity_from_psi_periodic_##SUF(T* u_z, T* u_r, T* psi, const T* R,     \
                                                      int nr, int nz, T dx, int ghost,        \
                                                      void* stream) {                         \
    axi::clear_error();                                                                       \
    AXI_TRY(axi::check_grid("velocity_from_psi_periodic", nr, nz));                           \
    AXI_TRY(axi::check_ptrs("velocity_from_psi_periodic", {u_z, u_r, psi, R},                  \
                            {"u_z", "u_r", "psi", "R"}));                                      \
    AXI_TRY(ghost_comm<T>(psi, nr, nz, ghost, false, T(0), dx, axi::as_stream(stream)));      \
    velocity_from_psi_kernel<T><<<grid2d(nr, nz), dim3(BX, BY), 0, axi::as_stream(stream)>>>( \
        u_z, u_r, psi, R, nr, nz, dx);                                                        \
    return axi::launch_status("velocity_from_psi_periodic");                                  \
  }

#define AXI_DEFINE_VORTICITY(SUF, T)                                                          \
  extern "C" int axi_vorticity_from_velocity_unb_##SUF(T* vort, const T* u_z, const T* u_r,   \
                                                       int nr, int nz, T dx, void* stream) {  \
    axi::clear_error();                                                                       \
    AXI_TRY(axi::check_grid("vorticity_from_velocity", nr, nz));                              \
    AXI_TRY(axi::check_ptrs("vorticity_from_velocity", {vort, u_z, u_r},                       \
                            {"vort", "u_z", "u_r"}));                                          \
    vorticity_from_velocity_kernel<T>                                                         \
        <<<grid2d(nr, nz), dim3(BX, BY), 0, axi::as_stream(stream)>>>(vort, u_z, u_r, nr, nz,  \
                                                                      dx);                    \
    return axi::launch_status("vorticity_from_velocity");                                     \
  }                                                                                           \
  extern "C" int axi_vorticity_from_velocity_periodic_##SUF(T* vort, T* u_z, T* u_r, int nr,  \
                                                            int nz, T dx, int ghost,          \
                                                            void* stream) {                   \
    axi::clear_error();                                                                       \
    AXI_TRY(axi::check_grid("vorticity_from_velocity_periodic", nr, nz));                     \
    AXI_TRY(axi::check_ptrs("vorticity_from_velocity_periodic", {vort, u_z, u_r},              \
                            {"vort", "u_z", "u_r"}));                                          \
    AXI_TRY(ghost_comm<T>(u_r, nr, nz, ghost, false, T(0), dx, axi::as_stream(stream)));      \
    AXI_TRY(ghost_comm<T>(u_z, nr, nz, ghost, false, T(0), dx, axi::as_stream(stream)));      \
    vorticity_from_velocity_kernel<T>                                                         \
        <<<grid2d(nr, nz), dim3(BX, BY), 0, axi::as_stream(stream)>>>(vort, u_z, u_r, nr, nz,  \
                                                                      dx);                    \
    return axi::launch_status("vorticity_from_velocity_periodic");                            \
  }

#define AXI_DEFINE_POINTWISE(SUF, T)                                                           \
  extern "C" int axi_brinkmann_penalize_##SUF(T lam, T dt, const T* chi, T U_z, T U_r,         \
                                              const T* gz, const T* gr, T* pz, T* pr,          \
                                              int64_t n, void* stream) {                       \
    axi::clear_error();                                                                        \
    if (n < 0) { axi::set_error("brinkmann_penalize: negative size"); return AXI_ERR_INVALID; } \
    if (n == 0) return AXI_OK;                                                                 \
    AXI_TRY(axi::check_ptrs("brinkmann_penalize", {chi, gz, gr, pz, pr},                       \
                            {"char_func", "grid_u_z", "grid_u_r", "penalized_u_z",             \
                             "penalized_u_r"}));                                               \
    brinkman_kernel<T><<<axi::ceil_div(n, 256), 256, 0, axi::as_stream(stream)>>>(            \
        lam, dt, chi, U_z, U_r, gz, gr, pz, pr, n);                                            \
    return axi::launch_status("brinkmann_penalize");                                          \
  }                                                                                            \
  extern "C" int axi_smooth_heaviside_##SUF(T* H, const T* phi, T w, int64_t n, void* stream) { \
    axi::clear_error();                                                                        \
    if (n < 0) { axi::set_error("smooth_heaviside: negative size"); return AXI_ERR_INVALID; }  \
    if (n == 0) return AXI_OK;                                                                 \
    AXI_TRY(axi::check_ptrs("smooth_heaviside", {H, phi}, {"H", "phi"}));                      \
    heaviside_kernel<T><<<axi::ceil_div(n, 256), 256, 0, axi::as_stream(stream)>>>(H, phi, w, n); \
    return axi::launch_status("smooth_heaviside");                                             \
  }                                                                                            \
  extern "C" int axi_kill_boundary_vorticity_sine_z_##SUF(T* vort, const T* Z, int nr, int nz, \
                                                          int width, T dx, void* stream) {     \
    axi::clear_error();                                                                        \
    if (width < 2 || width > 8 || 2 * width > nz || nr < 1) {                                  \
      axi::set_error("kill_boundary_vorticity_sine_z: width %d unsupported for nz = %d", width, nz); \
      return AXI_ERR_INVALID;                                                                  \
    }                                                                                          \
    AXI_TRY(axi::check_ptrs("kill_boundary_vorticity_sine_z", {vort, Z}, {"vorticity", "Z"})); \
    kill_z_kernel<T><<<axi::ceil_div(nr, 128), 128, 0, axi::as_stream(stream)>>>(vort, Z, nr, nz, \
                                                                                 width, dx);   \
    return axi::launch_status("kill_boundary_vorticity_sine_z");                               \
  }                                                                                            \
  extern "C" int axi_kill_boundary_vorticity_sine_r_##SUF(T* vort, const T* R, int nr, int nz, \
                                                          int width, T dx, void* stream) {     \
    axi::clear_error();                                                                        \
    if (width < 2 || width > nr || nz < 1) {                                                   \
      axi::set_error("kill_boundary_vorticity_sine_r: width %d unsupported for nr = %d", width, nr); \
      return AXI_ERR_INVALID;                                                                  \
    }                                                                                          \
    AXI_TRY(axi::check_ptrs("kill_boundary_vorticity_sine_r", {vort, R}, {"vorticity", "R"})); \
    kill_r_kernel<T><<<axi::ceil_div(nz, 128), 128, 0, axi::as_stream(stream)>>>(vort, R, nr, nz, \
                                                                                 width, dx);   \
    return axi::launch_status("kill_boundary_vorticity_sine_r");                               \
  }                                                                                            \
  extern "C" int axi_diffusion_rk2_unb_##SUF(T* vort, T* tmp, const T* R, int nr, int nz, T nu, \
                                             T dt, T dx, void* stream) {                       \
    axi::clear_error();                                                                        \
    AXI_TRY(axi::check_grid("diffusion_rk2", nr, nz));                                         \
    AXI_TRY(axi::check_ptrs("diffusion_rk2", {vort, tmp, R},                                   \
                            {"vorticity", "temp_vorticity", "R"}));                            \
    cudaStream_t s = axi::as_stream(stream);                                                   \
    const T dx2 = rn_host_mul(dx, dx), two_dx = rn_host_mul(T(2), dx);                         \
    const T c1 = rn_host_mul(rn_host_mul(T(0.5), nu), dt), c2 = rn_host_mul(nu, dt);           \
    rk2_stage1_kernel<T><<<grid2d(nr, nz), dim3(BX, BY), 0, s>>>(vort, tmp, R, nr, nz, c1, dx2, \
                                                                  two_dx);                     \
    rk2_stage2_kernel<T><<<grid2d(nr, nz), dim3(BX, BY), 0, s>>>(vort, tmp, R, nr, nz, c2, dx2, \
                                                                  two_dx);                     \
    return axi::launch_status("diffusion_rk2");                                                \
  }                                                                                            \
  extern "C" int axi_diffusion_rk2_periodic_##SUF(T* vort, T* tmp, const T* R, int nr, int nz, \
                                                  T nu, T dt, T dx, int ghost, void* stream) { \
    axi::clear_error();                                                                        \
    AXI_TRY(axi::check_grid("diffusion_rk2_periodic", nr, nz));                                \
    AXI_TRY(axi::check_ptrs("diffusion_rk2_periodic", {vort, tmp, R},                          \
                            {"vorticity", "temp_vorticity", "R"}));                            \
    cudaStream_t s = axi::as_stream(stream);                                                   \
    const T dx2 = rn_host_mul(dx, dx), two_dx = rn_host_mul(T(2), dx);                         \
    const T c1 = rn_host_mul(rn_host_mul(T(0.5), nu), dt), c2 = rn_host_mul(nu, dt);           \
    AXI_TRY(ghost_comm<T>(vort, nr, nz, ghost, false, T(0), dx, s));                           \
    rk2_stage1_kernel<T><<<grid2d(nr, nz), dim3(BX, BY), 0, s>>>(vort, tmp, R, nr, nz, c1, dx2, \
                                                                  two_dx);                     \
    AXI_TRY(ghost_comm<T>(tmp, nr, nz, ghost, false, T(0), dx, s));                            \
    rk2_stage2_kernel<T><<<grid2d(nr, nz), dim3(BX, BY), 0, s>>>(vort, tmp, R, nr, nz, c2, dx2, \
                                                                  two_dx);                     \
    return axi::launch_status("diffusion_rk2_periodic");                                       \
  }                                                                                            \
  extern "C" int axi_periodic_ghost_comm_##SUF(T* f, int nr, int nz, int ghost, void* stream) { \
    axi::clear_error();                                                                        \
    return ghost_comm<T>(f, nr, nz, ghost, false, T(0), T(0), axi::as_stream(stream));         \
  }                                                                                            \
  extern "C" int axi_periodic_ghost_comm_eta_##SUF(T* f, int nr, int nz, int ghost, T z_max,   \
                                                   T dx, void* stream) {                       \
    axi::clear_error();                                                                        \
    return ghost_comm<T>(f, nr, nz, ghost, true, z_max, dx, axi::as_stream(stream));           \
  }                                                                                            \
  extern "C" int axi_solid_sigma_##SUF(T* s11, T* s12, T* s22, T G, T dx, const T* e1,        \
                                       const T* e2, T* e1z, T* e1r, T* e2z, T* e2r, int nr,    \
                                       int nz, void* stream) {                                 \
    axi::clear_error();                                                                        \
    AXI_TRY(axi::check_grid("solid_sigma", nr, nz));                                           \
    AXI_TRY(axi::check_ptrs("solid_sigma", {s11, s12, s22, e1, e2, e1z, e1r, e2z, e2r},        \
                            {"sigma_11", "sigma_12", "sigma_22", "eta1", "eta2", "eta1_z",     \
                             "eta1_r", "eta2_z", "eta2_r"}));                                  \
    solid_sigma_kernel<T><<<grid2d(nr, nz), dim3(BX, BY), 0, axi::as_stream(stream)>>>(        \
        s11, s12, s22, G, dx, e1, e2, e1z, e1r, e2z, e2r, nr, nz);                             \
    return axi::launch_status("solid_sigma");                                                  \
  }                                                                                            \
  extern "C" int axi_update_vorticity_from_solid_stress_##SUF(                                 \
      T* vort, T* tau_z, T* tau_r, const T* t11, const T* t12, const T* t22, const T* R,       \
      int nr, int nz, T dt, T dx, void* stream) {                                              \
    axi::clear_error();                                                                        \
    AXI_TRY(axi::check_grid("update_vorticity_from_solid_stress", nr, nz));                    \
    AXI_TRY(axi::check_ptrs("update_vorticity_from_solid_stress",                              \
                            {vort, tau_z, tau_r, t11, t12, t22, R},                            \
                            {"vorticity", "tau_z", "tau_r", "sigma_11", "sigma_12",            \
                             "sigma_22", "R"}));                                               \
    cudaStream_t s = axi::as_stream(stream);                                                   \
    div_tau_kernel<T><<<grid2d(nr, nz), dim3(BX, BY), 0, s>>>(tau_z, tau_r, t11, t12, t22, R,  \
                                                               nr, nz, dx);                    \
    curl_tau_kernel<T><<<grid2d(nr, nz), dim3(BX, BY), 0, s>>>(vort, tau_z, tau_r, nr, nz, dt, \
                                                                dx);                           \
    return axi::launch_status("update_vorticity_from_solid_stress");                           \
  }

AXI_DEFINE_VELOCITY(f64, double)
AXI_DEFINE_VELOCITY(f32, float)
AXI_DEFINE_VORTICITY(f64, double)
AXI_DEFINE_VORTICITY(f32, float)
AXI_DEFINE_POINTWISE(f64, double)
AXI_DEFINE_POINTWISE(f32, float)

// The soft-sphere loop's dt-dependent kernels with the time step read on the
// device (state[AXI_SOFT_DT]); the arithmetic of the host-dt entries above.
extern "C" int axi_soft_update_vorticity_from_solid_stress_f64(
    double* vort, double* tau_z, double* tau_r, const double* t11, const double* t12,
    const double* t22, const double* R, int nr, int nz, double dx, const double* state,
    void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_grid("soft_update_vorticity_from_solid_stress", nr, nz));
  AXI_TRY(axi::check_ptrs("soft_update_vorticity_from_solid_stress",
                          {vort, tau_z, tau_r, t11, t12, t22, R, state},
                          {"vorticity", "tau_z", "tau_r", "sigma_11", "sigma_12", "sigma_22", "R",
                           "state"}));
  cudaStream_t s = axi::as_stream(stream);
  div_tau_kernel<double><<<grid2d(nr, nz), dim3(BX, BY), 0, s>>>(tau_z, tau_r, t11, t12, t22, R,
                                                                  nr, nz, dx);
  curl_tau_kernel<double><<<grid2d(nr, nz), dim3(BX, BY), 0, s>>>(vort, tau_z, tau_r, nr, nz,
                                                                   0.0, dx, state + AXI_SOFT_DT);
  return axi::launch_status("soft_update_vorticity_from_solid_stress");
}

extern "C" int axi_soft_diffusion_rk2_f64(double* vort, double* tmp, const double* R, int nr,
                                          int nz, double nu, double dx, const double* state,
                                          void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_grid("soft_diffusion_rk2", nr, nz));
  AXI_TRY(axi::check_ptrs("soft_diffusion_rk2", {vort, tmp, R, state},
                          {"vorticity", "temp_vorticity", "R", "state"}));
  cudaStream_t s = axi::as_stream(stream);
  const double dx2 = rn_host_mul(dx, dx), two_dx = rn_host_mul(2.0, dx);
  const double half_nu = rn_host_mul(0.5, nu);
  rk2_stage1_kernel<double><<<grid2d(nr, nz), dim3(BX, BY), 0, s>>>(
      vort, tmp, R, nr, nz, half_nu, dx2, two_dx, state + AXI_SOFT_DT);
  rk2_stage2_kernel<double><<<grid2d(nr, nz), dim3(BX, BY), 0, s>>>(
      vort, tmp, R, nr, nz, nu, dx2, two_dx, state + AXI_SOFT_DT);
  return axi::launch_status("soft_diffusion_rk2");
}
