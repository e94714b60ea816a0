// Fused per-timestep engine for flows past rigid bodies (one or many cases).
//
// One step is the loop body of examples/FlowPastSphere/flow_past_sphere.py:107-188:
//   kill boundary vorticity -> psi = Poisson^-1(r omega) -> u = curl(psi)/r +
//   free stream -> dt = min(diffusive, CFL) -> Brinkman penalisation ->
//   omega += curl(u_pen - u) -> drag -> ENO3 advection -> RK2 diffusion.
// Everything stays on the device: dt, the drag coefficient and the simulated
// time live in a per-case state block, so a step needs no host round trip and
// a run of steps can be captured in a CUDA graph.
//
// Launches per step (each covers every case of the plan):
//   kill_reset   one block per case: sine tapers, state reset
//   transform    four dense products per case (spectral Poisson solve)
//   vel_max      per tile: velocity, max(|u_z| + |u_r|) -> atomicMax
//   penalise     per tile: velocity + Brinkman + curl(u_pen - u) into omega,
//                drag partials; the last tile of a case finalises dt/Cd/t
//   adv_diff1    per tile: ENO3 advection (axis mirror by index reflection,
//                halo 3 in shared memory) + RK2 stage 1
//   diff2        per tile: RK2 stage 2 into omega
// Arithmetic uses FMA and precomputed reciprocals (1 / (2 dx r), 1 / r^2);
// parity with the reference is to a relative L2 of 1e-12 after N steps in
// FP64. Reductions (max, drag) are order-independent or in a fixed order.
#include "axi_common.cuh"
#include "gemm_simt.cuh"

namespace {

constexpr int TX = 32;
constexpr int TY = 8;
constexpr int NT = TX * TY;

struct TileRec {
  int c, i0, j0, idx;  // case, first row, first column, tile index within the case
};

template <typename T>
__device__ __forceinline__ T* F(void* p) {
  return static_cast<T*>(p);
}
template <typename T>
__device__ __forceinline__ const T* CF(const void* p) {
  return static_cast<const T*>(p);
}

__device__ __forceinline__ double ramp_prefac(const axi_case& k, double t) {
  // examples/FlowPastSphere/flow_past_sphere.py:118-121
  if (k.t_ramp > 0.0 && t < k.t_ramp) return sin(0.5 * 3.141592653589793 * t / k.t_ramp);
  return 1.0;
}

__device__ __forceinline__ double step_dt(const axi_case& k) {
  // flow_past_sphere.py:150-153: min(0.9 dx^2 / 4 / nu, CFL dx / (max|u| + eps))
  const double umax = __longlong_as_double(
      (long long)*reinterpret_cast<const unsigned long long*>(&k.state[AXI_ST_UMAX]));
  const double cfl_dt = (k.cfl * k.dx) / (umax + k.eps);
  return fmin(k.dt_diff, cfl_dt);
}

// d(psi)/dr * 1 / (2 dx) at (i, j) with one-sided rows at the axis and the
// outer boundary (kernels/compute_velocity_from_psi.py:10-12), in double.
template <typename T, typename Acc>
__device__ __forceinline__ double dpsi_dr(Acc psi, int i, int j, int nr) {
  if (i == 0) return -(double)psi(2, j) + 4.0 * (double)psi(1, j) - 3.0 * (double)psi(0, j);
  if (i == nr - 1)
    return (double)psi(nr - 3, j) - 4.0 * (double)psi(nr - 2, j) + 3.0 * (double)psi(nr - 1, j);
  return (double)psi(i + 1, j) - (double)psi(i - 1, j);
}

template <typename T, typename Acc>
__device__ __forceinline__ double dpsi_dz(Acc psi, int i, int j, int nz) {
  if (j == 0) return -(double)psi(i, 2) + 4.0 * (double)psi(i, 1) - 3.0 * (double)psi(i, 0);
  if (j == nz - 1)
    return (double)psi(i, nz - 3) - 4.0 * (double)psi(i, nz - 2) + 3.0 * (double)psi(i, nz - 1);
  return (double)psi(i, j + 1) - (double)psi(i, j - 1);
}

// ---------------------------------------------------------------------------
// kill_reset: kernels/kill_boundary_vorticity_sine.py:4-27 (literal 1 - Z,
// 1 - R), then clear the per-step reduction words.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void kill_reset_kernel(const axi_case* __restrict__ cases) {
  const axi_case& k = cases[blockIdx.x];
  T* w = F<T>(k.omega);
  const int nr = k.nr, nz = k.nz, wd = k.kill_width;
  const double dx = k.dx, half_dx = 0.5 * k.dx;
  const double pi = 3.141592653589793;
  if (threadIdx.x == 0) {
    *reinterpret_cast<unsigned long long*>(&k.state[AXI_ST_UMAX]) = 0ull;
    *reinterpret_cast<unsigned int*>(&k.state[AXI_ST_COUNT]) = 0u;
  }
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    T* row = w + (long long)i * nz;
    const double left = (double)row[wd - 1];
    double nl[8];
    for (int q = 0; q < wd; ++q) nl[q] = sin(pi * (k.z[q] - half_dx) / 2 / (wd - 1) / dx) * left;
    for (int q = 0; q < wd; ++q) row[q] = (T)nl[q];
    const double right = (double)row[nz - wd];
    for (int q = 0; q < wd; ++q)
      nl[q] = sin(pi * (1 - k.z[nz - wd + q] - half_dx) / 2 / (wd - 1) / dx) * right;
    for (int q = 0; q < wd; ++q) row[nz - wd + q] = (T)nl[q];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nz; j += blockDim.x) {
    const double src = (double)w[(long long)(nr - wd) * nz + j];
    for (int q = 0; q < wd; ++q) {
      const int i = nr - wd + q;
      w[(long long)i * nz + j] = (T)(sin(pi * (1 - k.r[i] - half_dx) / 2 / (wd - 1) / dx) * src);
    }
    w[j] = T(0);
  }
}

// ---------------------------------------------------------------------------
// vel_max: max over the case of |u_z| + |u_r| (flow_past_sphere.py:152)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(NT) vel_max_kernel(const axi_case* __restrict__ cases,
                                                     const int4* __restrict__ tiles) {
  const int4 tr = tiles[blockIdx.x];
  const axi_case& k = cases[tr.x];
  const int i = tr.y + threadIdx.x / TX;
  const int j = tr.z + threadIdx.x % TX;
  const int nr = k.nr, nz = k.nz;
  const T* psi = CF<T>(k.psi);
  double v = 0.0;
  if (i < nr && j < nz) {
    auto acc = [&](int a, int b) { return psi[(long long)a * nz + b]; };
    const double prefac = ramp_prefac(k, k.state[AXI_ST_T]);
    const double uz = (double)(T)(dpsi_dr<T>(acc, i, j, nr) * k.rinv2dx[i]) + k.U0 * prefac;
    const double ur = (double)(T)(-dpsi_dz<T>(acc, i, j, nz) * k.rinv2dx[i]);
    v = fabs((double)(T)uz) + fabs(ur);
  }
  // block max (NaN propagates: its bit pattern compares above +inf)
  unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long other = __shfl_down_sync(0xffffffffu, bits, o);
    bits = other > bits ? other : bits;
  }
  __shared__ unsigned long long wmax[NT / 32];
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = bits;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = 0;
    for (int q = 0; q < NT / 32; ++q) m = wmax[q] > m ? wmax[q] : m;
    atomicMax(reinterpret_cast<unsigned long long*>(&k.state[AXI_ST_UMAX]), m);
  }
}

// ---------------------------------------------------------------------------
// penalise: flow_past_sphere.py:156-175 (Brinkman, penalisation vorticity, drag)
// ---------------------------------------------------------------------------
// Penalised velocity at (gi, gj): u from psi (plus the ramped free stream),
// then (u + lam dt chi U_body) / (1 + lam dt chi) (kernels/brinkmann_penalize.py:11-16).
template <typename T, typename Acc>
__device__ __forceinline__ void penalised_velocity(const axi_case& k, Acc psi, int gi, int gj,
                                                   double prefac, double lamdt, T chi, T& uz,
                                                   T& ur, T& pz, T& pr) {
  const double drv = dpsi_dr<T>(psi, gi, gj, k.nr);
  const double dzv = dpsi_dz<T>(psi, gi, gj, k.nz);
  const double rinv = k.rinv2dx[gi];
  uz = (T)((double)(T)(drv * rinv) + k.U0 * prefac);
  ur = (T)(-dzv * rinv);
  const double lc = lamdt * (double)chi;
  const double inv = 1.0 / (1.0 + lc);
  pz = (T)(((double)uz + lc * k.U_body) * inv);
  pr = (T)((double)ur * inv);
}

template <typename T>
__global__ void __launch_bounds__(NT) penalise_kernel(const axi_case* __restrict__ cases,
                                                      const int4* __restrict__ tiles) {
  __shared__ T ps[TY + 4][TX + 4];
  __shared__ T duz[TY + 2][TX + 2];
  __shared__ T dur[TY + 2][TX + 2];
  __shared__ double red[NT / 32];
  __shared__ bool last;
  const int4 tr = tiles[blockIdx.x];
  const axi_case& k = cases[tr.x];
  const int nr = k.nr, nz = k.nz;
  const int i0 = tr.y, j0 = tr.z;
  const T* psi = CF<T>(k.psi);
  const T* chi = CF<T>(k.chi);
  const double dt = step_dt(k);
  const double prefac = ramp_prefac(k, k.state[AXI_ST_T]);
  const double lamdt = k.lam * dt;
  // psi tile with halo 2 (every one-sided boundary stencil stays inside it)
  for (int e = threadIdx.x; e < (TY + 4) * (TX + 4); e += NT) {
    const int a = e / (TX + 4), b = e % (TX + 4);
    const int gi = i0 - 2 + a, gj = j0 - 2 + b;
    ps[a][b] = (gi >= 0 && gi < nr && gj >= 0 && gj < nz) ? psi[(long long)gi * nz + gj] : T(0);
  }
  __syncthreads();
  auto sp = [&](int gi, int gj) { return ps[gi - i0 + 2][gj - j0 + 2]; };
  // u_pen - u on the tile and a one-cell halo
  for (int e = threadIdx.x; e < (TY + 2) * (TX + 2); e += NT) {
    const int a = e / (TX + 2), b = e % (TX + 2);
    const int gi = i0 - 1 + a, gj = j0 - 1 + b;
    T dz = T(0), dr = T(0);
    if (gi >= 0 && gi < nr && gj >= 0 && gj < nz) {
      T uz, ur, pz, pr;
      penalised_velocity<T>(k, sp, gi, gj, prefac, lamdt, chi[(long long)gi * nz + gj], uz, ur,
                            pz, pr);
      dz = pz - uz;
      dr = pr - ur;
    }
    duz[a][b] = dz;
    dur[a][b] = dr;
  }
  __syncthreads();
  double cd_part = 0.0;
  {
    const int a = threadIdx.x / TX, b = threadIdx.x % TX;
    const int gi = i0 + a, gj = j0 + b;
    if (gi < nr && gj < nz) {
      const long long c = (long long)gi * nz + gj;
      const T ch = chi[c];
      T uz, ur, pz, pr;
      penalised_velocity<T>(k, sp, gi, gj, prefac, lamdt, ch, uz, ur, pz, pr);
      F<T>(k.u_z)[c] = pz;
      F<T>(k.u_r)[c] = pr;
      // drag integrand R chi u_z (flow_past_sphere.py:173), FP64
      cd_part = k.r[gi] * (double)ch * (double)pz;
      if (gi >= 1 && gi < nr - 1 && gj >= 1 && gj < nz - 1) {
        // compute_vorticity_from_velocity.py:11-13 on u_pen - u
        const T inv2dx = (T)(0.5 / k.dx);
        const T pw = (dur[a + 1][b + 2] - dur[a + 1][b]) * inv2dx -
                     (duz[a + 2][b + 1] - duz[a][b + 1]) * inv2dx;
        T* w = F<T>(k.omega);
        w[c] = w[c] + pw;
      }
    }
  }
  // drag: tile sum in a fixed order (warp shuffles, then warps in order)
  double x = cd_part;
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  const unsigned int ntiles = (unsigned int)(((nr + TY - 1) / TY) * ((nz + TX - 1) / TX));
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int q = 0; q < NT / 32; ++q) sum += red[q];
    k.partials[tr.w] = sum;
    __threadfence();
    const unsigned int done =
        atomicAdd(reinterpret_cast<unsigned int*>(&k.state[AXI_ST_COUNT]), 1u);
    last = (done == ntiles - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    // last tile of the case: case totals in tile order, then dt / Cd
    __threadfence();
    double sum = 0.0;
    for (unsigned int q = 0; q < ntiles; ++q) sum += ((volatile double*)k.partials)[q];
    const double cd = k.cd_scale * sum;
    const double umax = __longlong_as_double(
        (long long)*reinterpret_cast<const unsigned long long*>(&k.state[AXI_ST_UMAX]));
    if (!(umax <= 1.7976931348623157e308) || !(cd == cd))
      atomicOr(reinterpret_cast<unsigned int*>(&k.state[AXI_ST_STATUS]), 1u << AXI_ERR_NONFINITE);
    const long long step = (long long)k.state[AXI_ST_STEPS];
    if (k.history && step < k.history_len) {
      k.history[2 * step] = dt;
      k.history[2 * step + 1] = cd;
    }
    k.state[AXI_ST_CD] = cd;
    k.state[AXI_ST_DT] = dt;
    k.state[AXI_ST_FORCE] = sum;
  }
}

// ---------------------------------------------------------------------------
// adv_diff1: ENO3 advection (kernels/advect_vorticity_via_eno3.py:28-42,
// pyst_kernels/advection_flux.py:9-163, advection_timestep.py:37-54) and RK2
// stage 1 (kernels/diffusion_RK2.py:9-26)
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T face_flux(T fm1, T f0, T f1, T f2, T um1, T u0, T u1, T u2) {
  const T third = T(1) / T(3), five6 = T(5) / T(6), sixth = T(1) / T(6);
  if (u0 > -u1) return third * f1 * u1 + five6 * f0 * u0 - sixth * fm1 * um1;
  return third * f0 * u0 + five6 * f1 * u1 - sixth * f2 * u2;
}

template <typename T>
__global__ void __launch_bounds__(NT) adv_diff1_kernel(const axi_case* __restrict__ cases,
                                                       const int4* __restrict__ tiles) {
  constexpr int H = 3;
  __shared__ T sw[TY + 2 * H][TX + 2 * H];
  __shared__ T sz[TY + 2 * H][TX + 2 * H];
  __shared__ T sr[TY + 2 * H][TX + 2 * H];
  __shared__ T wa[TY + 2][TX + 2];
  const int4 tr = tiles[blockIdx.x];
  const axi_case& k = cases[tr.x];
  const int nr = k.nr, nz = k.nz;
  const int i0 = tr.y, j0 = tr.z;
  const T* w = CF<T>(k.omega);
  const T* uz = CF<T>(k.u_z);
  const T* ur = CF<T>(k.u_r);
  const double dt = k.state[AXI_ST_DT];
  const T a = (T)(-dt / k.dx);
  for (int e = threadIdx.x; e < (TY + 2 * H) * (TX + 2 * H); e += NT) {
    const int p = e / (TX + 2 * H), q = e % (TX + 2 * H);
    const int gi = i0 - H + p, gj = j0 - H + q;
    T vw = T(0), vz = T(0), vr = T(0);
    if (gj >= 0 && gj < nz && gi < nr) {
      if (gi >= 0) {
        const long long c = (long long)gi * nz + gj;
        vw = w[c];
        vz = uz[c];
        vr = ur[c];
      } else if (-1 - gi < nr) {
        // rows below the axis: omega odd, u_z even, u_r odd
        const long long c = (long long)(-1 - gi) * nz + gj;
        vw = -w[c];
        vz = uz[c];
        vr = -ur[c];
      }
    }
    sw[p][q] = vw;
    sz[p][q] = vz;
    sr[p][q] = vr;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < (TY + 2) * (TX + 2); e += NT) {
    const int p = e / (TX + 2), q = e % (TX + 2);
    const int gi = i0 - 1 + p, gj = j0 - 1 + q;
    T val = T(0);
    if (gi >= 0 && gi < nr && gj >= 0 && gj < nz) {
      const int P = p + H - 1, Q = q + H - 1;  // position in the halo-3 tiles
      const T f0 = sw[P][Q];
      T flux = T(0);
      if (gi < nr - 2 && gj >= 2 && gj < nz - 2) {
        const T xf = face_flux(sw[P][Q - 1], f0, sw[P][Q + 1], sw[P][Q + 2], sz[P][Q - 1],
                               sz[P][Q], sz[P][Q + 1], sz[P][Q + 2]);
        const T xb = face_flux(sw[P][Q - 2], sw[P][Q - 1], f0, sw[P][Q + 1], sz[P][Q - 2],
                               sz[P][Q - 1], sz[P][Q], sz[P][Q + 1]);
        const T yf = face_flux(sw[P - 1][Q], f0, sw[P + 1][Q], sw[P + 2][Q], sr[P - 1][Q],
                               sr[P][Q], sr[P + 1][Q], sr[P + 2][Q]);
        const T yb = face_flux(sw[P - 2][Q], sw[P - 1][Q], f0, sw[P + 1][Q], sr[P - 2][Q],
                               sr[P - 1][Q], sr[P][Q], sr[P + 1][Q]);
        flux = a * xf;
        flux = flux - a * xb;
        flux = flux + a * yf;
        flux = flux - a * yb;
      }
      val = f0 + flux;
    }
    wa[p][q] = val;
  }
  __syncthreads();
  const int p = threadIdx.x / TX, q = threadIdx.x % TX;
  const int gi = i0 + p, gj = j0 + q;
  if (gi < nr && gj < nz) {
    const T c0 = wa[p + 1][q + 1];
    T tmp = c0;
    if (gi >= 1 && gi < nr - 1 && gj >= 1 && gj < nz - 1) {
      const T n = wa[p + 2][q + 1], s = wa[p][q + 1], e = wa[p + 1][q + 2], ww = wa[p + 1][q];
      const T inv_dx2 = (T)(1.0 / (k.dx * k.dx));
      const T lap = (n + s + e + ww - T(4) * c0) * inv_dx2 + (n - s) * (T)k.rinv2dx[gi] -
                    c0 * (T)k.rinv2[gi];
      tmp = c0 + (T)(0.5 * k.nu * dt) * lap;
    }
    const long long c = (long long)gi * nz + gj;
    F<T>(k.w_adv)[c] = c0;
    F<T>(k.w_tmp)[c] = tmp;
  }
}

// ---------------------------------------------------------------------------
// diff2: RK2 stage 2 (kernels/diffusion_RK2.py:27-44); advances the time
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(NT) diff2_kernel(const axi_case* __restrict__ cases,
                                                   const int4* __restrict__ tiles) {
  const int4 tr = tiles[blockIdx.x];
  const axi_case& k = cases[tr.x];
  const int nr = k.nr, nz = k.nz;
  const int gi = tr.y + threadIdx.x / TX, gj = tr.z + threadIdx.x % TX;
  const double dt = k.state[AXI_ST_DT];
  if (gi < nr && gj < nz) {
    const long long c = (long long)gi * nz + gj;
    const T* wa = CF<T>(k.w_adv);
    const T* tm = CF<T>(k.w_tmp);
    T v = wa[c];
    if (gi >= 1 && gi < nr - 1 && gj >= 1 && gj < nz - 1) {
      const T c0 = tm[c], n = tm[c + nz], s = tm[c - nz], e = tm[c + 1], ww = tm[c - 1];
      const T inv_dx2 = (T)(1.0 / (k.dx * k.dx));
      const T lap = (n + s + e + ww - T(4) * c0) * inv_dx2 + (n - s) * (T)k.rinv2dx[gi] -
                    c0 * (T)k.rinv2[gi];
      v = v + (T)(k.nu * dt) * lap;
    }
    F<T>(k.omega)[c] = v;
  }
  if (tr.w == 0 && threadIdx.x == 0) {
    k.state[AXI_ST_T] += dt;
    k.state[AXI_ST_STEPS] += 1.0;
  }
}

inline int tiles_of(const axi_case& k) { return ((k.nr + TY - 1) / TY) * ((k.nz + TX - 1) / TX); }

// Phases of one step, in launch order.
enum { PH_KILL = 0, PH_TRANSFORM = 1, PH_VEL_MAX = 2, PH_PENALISE = 3, PH_ADV_DIFF1 = 4,
       PH_DIFF2 = 5, PH_COUNT = 6 };

template <typename T>
int run_phase(int phase, const axi_case* hcases, int n_cases, const axi_case* dcases,
              const int4* tiles, int n_tiles, cudaStream_t s) {
  switch (phase) {
    case PH_KILL:
      kill_reset_kernel<T><<<n_cases, 256, 0, s>>>(dcases);
      break;
    case PH_TRANSFORM:
      for (int c = 0; c < n_cases; ++c) {
        const axi_case& k = hcases[c];
        AXI_TRY(axi_gemm::fd_transform<T>(
            static_cast<T*>(k.psi), k.nz, static_cast<const T*>(k.omega), k.nz,
            static_cast<const T*>(k.Er_inv_w), static_cast<const T*>(k.EzinvT),
            static_cast<const T*>(k.inv_eig), static_cast<const T*>(k.Er),
            static_cast<const T*>(k.EzT), static_cast<T*>(k.gemm_work), k.nr, k.nz, s));
      }
      break;
    case PH_VEL_MAX:
      vel_max_kernel<T><<<n_tiles, NT, 0, s>>>(dcases, tiles);
      break;
    case PH_PENALISE:
      penalise_kernel<T><<<n_tiles, NT, 0, s>>>(dcases, tiles);
      break;
    case PH_ADV_DIFF1:
      adv_diff1_kernel<T><<<n_tiles, NT, 0, s>>>(dcases, tiles);
      break;
    case PH_DIFF2:
      diff2_kernel<T><<<n_tiles, NT, 0, s>>>(dcases, tiles);
      break;
    default:
      axi::set_error("rigid_phase: unknown phase %d", phase);
      return AXI_ERR_INVALID;
  }
  return axi::launch_status("rigid_phase");
}

inline const int4* tile_table(const void* plan_dev, int n_cases) {
  return reinterpret_cast<const int4*>(static_cast<const char*>(plan_dev) +
                                       ((n_cases * sizeof(axi_case) + 15) & ~size_t(15)));
}

template <typename T>
int rigid_step(const axi_case* hcases, int n_cases, const void* plan_dev, int n_tiles,
               int n_steps, cudaStream_t s, const char* what) {
  const axi_case* dcases = static_cast<const axi_case*>(plan_dev);
  const int4* tiles = tile_table(plan_dev, n_cases);
  for (int step = 0; step < n_steps; ++step)
    for (int ph = 0; ph < PH_COUNT; ++ph)
      AXI_TRY(run_phase<T>(ph, hcases, n_cases, dcases, tiles, n_tiles, s));
  return axi::launch_status(what);
}

int validate(const axi_case* cases, int n_cases, const char* what) {
  if (n_cases <= 0 || n_cases > 65535) {
    axi::set_error("%s: invalid case count %d", what, n_cases);
    return AXI_ERR_INVALID;
  }
  for (int c = 0; c < n_cases; ++c) {
    const axi_case& k = cases[c];
    if (k.nr < 8 || k.nz < 8 || k.kill_width < 2 || k.kill_width > 8 || 2 * k.kill_width > k.nz ||
        k.kill_width > k.nr) {
      axi::set_error("%s: case %d has an unsupported grid %d x %d / kill width %d", what, c, k.nr,
                     k.nz, k.kill_width);
      return AXI_ERR_INVALID;
    }
    const void* ptrs[] = {k.omega, k.psi, k.u_z, k.u_r, k.chi, k.w_adv, k.w_tmp, k.r, k.z,
                          k.rinv2dx, k.rinv2, k.Er, k.Er_inv_w, k.EzinvT, k.EzT, k.inv_eig,
                          k.gemm_work, k.state, k.partials};
    for (const void* p : ptrs) {
      if (!p) {
        axi::set_error("%s: case %d has a null pointer", what, c);
        return AXI_ERR_INVALID;
      }
    }
  }
  return AXI_OK;
}

}  // namespace

extern "C" int axi_plan_init(axi_case* cases, int n_cases, int64_t* plan_bytes, int* n_tiles) {
  axi::clear_error();
  AXI_TRY(validate(cases, n_cases, "plan_init"));
  int total = 0;
  for (int c = 0; c < n_cases; ++c) {
    cases[c].stencil_tile0 = total;
    total += tiles_of(cases[c]);
  }
  *n_tiles = total;
  *plan_bytes = (int64_t)(((n_cases * sizeof(axi_case) + 15) & ~size_t(15)) + total * sizeof(int4));
  return AXI_OK;
}

extern "C" int axi_plan_upload(const axi_case* cases, int n_cases, void* plan_dev, void* stream) {
  axi::clear_error();
  AXI_TRY(validate(cases, n_cases, "plan_upload"));
  AXI_TRY(axi::check_ptr("plan_upload", plan_dev, "plan_dev"));
  int total = 0;
  for (int c = 0; c < n_cases; ++c) total += tiles_of(cases[c]);
  const size_t head = (n_cases * sizeof(axi_case) + 15) & ~size_t(15);
  std::string buf(head + total * sizeof(int4), '\0');
  memcpy(&buf[0], cases, n_cases * sizeof(axi_case));
  int4* t = reinterpret_cast<int4*>(&buf[head]);
  int q = 0;
  for (int c = 0; c < n_cases; ++c) {
    const axi_case& k = cases[c];
    int idx = 0;
    for (int i0 = 0; i0 < k.nr; i0 += TY)
      for (int j0 = 0; j0 < k.nz; j0 += TX) t[q++] = make_int4(c, i0, j0, idx++);
  }
  cudaStream_t s = axi::as_stream(stream);
  if (cudaMemcpyAsync(plan_dev, buf.data(), buf.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return axi::launch_status("plan_upload");
  return AXI_OK;
}

extern "C" int axi_rigid_step_f64(const axi_case* cases, int n_cases, const void* plan_dev,
                                  int n_tiles, int n_steps, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("rigid_step", plan_dev, "plan_dev"));
  return rigid_step<double>(cases, n_cases, plan_dev, n_tiles, n_steps, axi::as_stream(stream),
                            "rigid_step_f64");
}

extern "C" int axi_rigid_step_f32(const axi_case* cases, int n_cases, const void* plan_dev,
                                  int n_tiles, int n_steps, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("rigid_step", plan_dev, "plan_dev"));
  return rigid_step<float>(cases, n_cases, plan_dev, n_tiles, n_steps, axi::as_stream(stream),
                           "rigid_step_f32");
}

extern "C" int axi_rigid_phase_f64(const axi_case* cases, int n_cases, const void* plan_dev,
                                   int n_tiles, int phase, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("rigid_phase", plan_dev, "plan_dev"));
  return run_phase<double>(phase, cases, n_cases, static_cast<const axi_case*>(plan_dev),
                           tile_table(plan_dev, n_cases), n_tiles, axi::as_stream(stream));
}

extern "C" int axi_rigid_phase_f32(const axi_case* cases, int n_cases, const void* plan_dev,
                                   int n_tiles, int phase, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("rigid_phase", plan_dev, "plan_dev"));
  return run_phase<float>(phase, cases, n_cases, static_cast<const axi_case*>(plan_dev),
                          tile_table(plan_dev, n_cases), n_tiles, axi::as_stream(stream));
}
