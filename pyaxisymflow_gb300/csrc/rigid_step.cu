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
// Launches per step, each covering every case of the plan:
//   kill_reset   one block per case: sine tapers, free stream of this step,
//                counters cleared, float copies of the step scalars
//   transform    four grouped dense products (the spectral Poisson solve)
//   vel_max      persistent, per tile: max(|u_z| + |u_r|) into the case
//   step_dt      one thread per case: dt and the dt-dependent constants
//   penalise     per tile: velocity + Brinkman + omega + curl(u_pen - u)
//                into the staging half of the work buffer, drag partials;
//                the last tile of a case finalises the drag
//   advect_diffuse per tile: ENO3 advection (axis mirror) and both RK2
//                stages in shared memory (halo 4) from the staged omega
//                into omega; advances the time
//                (sedimenting cases: mask rebuild, drag, body ODE)
// The stencil kernels receive their halo boxes by TMA.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the FP32 engine
// keeps every per-cell operation in FP32: per-row factors (1 / (2 dx r),
// 1 / r^2, r) are precomputed vectors in the engine precision and the
// per-step scalars are computed once per case. FP64 remains in the time
// step, the simulated time, the drag sums across warps and tiles and the
// body ODE.
#include <algorithm>
#include <type_traits>
#include <vector>

#include "axi_common.cuh"
#include "dct.cuh"
#include "dct64.cuh"
#include "tc_gemm.cuh"
#include "tma.cuh"

namespace {

// Stencil tiles: 64 x 32 cells per 256-thread block (8 cells per thread,
// warps along the contiguous z axis). Thread t owns column t % 64 of the tile
// and rows t / 64 + 4 m (m < 8); vel_max gives each thread 8 consecutive rows
// instead. Cell indices are 32-bit (a case has fewer than 2^31 cells).
constexpr int TX = AXI_TILE_NZ;
constexpr int TY = AXI_TILE_NR;
constexpr int NT = 256;
constexpr int CPT = TX * TY / NT;
constexpr int RG = NT / TX;  // row groups
static_assert(TX == 64 && TY % RG == 0, "tile shape");
constexpr double kPi = 3.141592653589793;

// Per-step scalars as the per-cell code reads them. The double engine reads
// the state words and case fields directly; the float engine reads float
// copies that kill_reset and vel_max write once per case and step, so no
// thread converts from double (GB300 issues FP64 conversions at the FP64
// rate).
// The float engine's body geometry is kept in cell units, split into float
// hi / lo pairs: S = z_cm / dx, R = radius / dx (and W = blend width / dx), so
// the moving mask sees the double position, not its float rounding.
enum {
  SF_UFREE, SF_LAMDT, SF_ADV, SF_C1, SF_C2, SF_UBODY, SF_INV2DX, SF_INVDX2,
  SF_S_HI, SF_S_LO, SF_R_HI, SF_R_LO, SF_W, SF_UBODY_LO, SF_FLOAT_END,
  // read by the double engine only (from the state block and the case)
  SF_ZCM = SF_FLOAT_END, SF_RBODY, SF_BLENDW
};
static_assert(SF_FLOAT_END <= 2 * (AXI_ST_WORDS - AXI_ST_F32), "float scalar slots");

// Tensor maps of a case's fields (the stencil kernels' TMA boxes) and the
// error codes of their bounded waits (plan error word).
enum { MAP_PSI = 0, MAP_CHI = 1, MAP_W = 2, MAP_UZ = 3, MAP_UR = 4, MAP_PSI_LO = 5, MAP_COUNT = 6 };
enum { ERR_STENCIL_WAIT = 5, ERR_STENCIL_DRAIN = 6 };

__device__ __forceinline__ float* fslots(const axi_case& k) {
  return reinterpret_cast<float*>(&k.state[AXI_ST_F32]);
}

template <typename T>
__device__ __forceinline__ T scalar(const axi_case& k, int f);
template <>
__device__ __forceinline__ float scalar<float>(const axi_case& k, int f) {
  return fslots(k)[f];  // f < SF_FLOAT_END
}
template <>
__device__ __forceinline__ double scalar<double>(const axi_case& k, int f) {
  switch (f) {
    case SF_UFREE: return k.state[AXI_ST_UFREE];
    case SF_LAMDT: return k.state[AXI_ST_LAMDT];
    case SF_ADV: return k.state[AXI_ST_ADV];
    case SF_C1: return k.state[AXI_ST_C1];
    case SF_C2: return k.state[AXI_ST_C2];
    case SF_UBODY:
      return (k.flags & AXI_CASE_SEDIMENTING) ? k.state[AXI_ST_UBODY] : k.U_body;
    case SF_ZCM: return k.state[AXI_ST_ZCM];
    case SF_INV2DX: return k.inv_2dx;
    case SF_INVDX2: return k.inv_dx2;
    case SF_RBODY: return k.r_body;
    default: return k.blend_w;
  }
}

template <typename T>
__device__ __forceinline__ T* F(void* p) {
  return static_cast<T*>(p);
}
template <typename T>
__device__ __forceinline__ const T* CF(const void* p) {
  return static_cast<const T*>(p);
}

__device__ __forceinline__ unsigned int* counter(const axi_case& k, int which) {
  return reinterpret_cast<unsigned int*>(&k.state[AXI_ST_COUNT]) + which;
}

// Keeps the TF32 hi / lo copy of omega (operand of the tensor-core products)
// in step with omega in the FP32 engine.
template <typename T>
__device__ __forceinline__ void store_omega(const axi_case& k, int c, T v) {
  F<T>(k.omega)[c] = v;
  if constexpr (sizeof(T) == 4) {
    if (k.omega_hi) {
      float hi, lo;
      axi_tc::tf32_split((float)v, hi, lo);
      static_cast<float*>(k.omega_hi)[c] = hi;
      static_cast<float*>(k.omega_lo)[c] = lo;
    }
  }
}

inline int tiles_of(const axi_case& k) { return ((k.nr + TY - 1) / TY) * ((k.nz + TX - 1) / TX); }
__device__ __forceinline__ unsigned int dev_tiles_of(const axi_case& k) {
  return (unsigned int)(((k.nr + TY - 1) / TY) * ((k.nz + TX - 1) / TX));
}

// ---------------------------------------------------------------------------
// kill_reset: kernels/kill_boundary_vorticity_sine.py:4-27 (literal 1 - Z,
// 1 - R), the ramped free stream (flow_past_sphere.py:118-121), counters.
//
// The z-edge taper of every row, then the outer-r taper of rows nr - w ..
// nr - 1 from row nr - w (itself z-tapered first), then row 0 set to zero,
// computed as one map of the incoming omega. Each output depends only on
// incoming values that its own thread reads before writing, except the two
// z-taper sources of row nr - w (columns w - 1 and nz - w), which all 2w
// edge columns of the outer rows read and two of them overwrite: those edge
// columns are threads of block 0 that read before a barrier and write after
// it. Work units of a case: the 2w edge columns, the nz - 2w inner columns
// (outer rows and row 0), rows 1 .. nr - w - 1 (their two z strips).
// ---------------------------------------------------------------------------
constexpr int KILL_BLOCKS = 4;  // blocks per case (grid x)

template <typename T>
__global__ void __launch_bounds__(256) kill_reset_kernel(const axi_case* __restrict__ cases,
                                                         unsigned int* __restrict__ vm_done) {
  const axi_case& k = cases[blockIdx.y];
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *vm_done = 0u;  // vel_max arrivals
  T* w = F<T>(k.omega);
  const int nr = k.nr, nz = k.nz, wd = k.kill_width;
  // taper factors sin(pi (Z - dx/2) / 2 / (w - 1) / dx) etc., evaluated once on
  // the host with the reference's own formula
  const double* cz0 = k.kill_coef;
  const double* cz1 = k.kill_coef + wd;
  const double* cr = k.kill_coef + 2 * wd;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *reinterpret_cast<unsigned long long*>(&k.state[AXI_ST_UMAX]) = 0ull;
    counter(k, 0)[0] = 0u;
    counter(k, 1)[0] = 0u;
    const double t = k.state[AXI_ST_T];
    double prefac = 1.0;
    if (k.t_ramp > 0.0 && t < k.t_ramp) prefac = sin(0.5 * kPi * t / k.t_ramp);
    k.state[AXI_ST_UFREE] = k.U0 * prefac;
    float* f = fslots(k);
    f[SF_UFREE] = (float)(k.U0 * prefac);
    const double ub = (k.flags & AXI_CASE_SEDIMENTING) ? k.state[AXI_ST_UBODY] : k.U_body;
    f[SF_UBODY] = (float)ub;
    f[SF_UBODY_LO] = (float)(ub - (double)(float)ub);  // the body velocity as a float pair
    f[SF_INV2DX] = (float)k.inv_2dx;
    f[SF_INVDX2] = (float)k.inv_dx2;
    const double sc = k.state[AXI_ST_ZCM] / k.dx, rc = k.r_body / k.dx;
    f[SF_S_HI] = (float)sc;
    f[SF_S_LO] = (float)(sc - (double)(float)sc);
    f[SF_R_HI] = (float)rc;
    f[SF_R_LO] = (float)(rc - (double)(float)rc);
    f[SF_W] = (float)(k.blend_w / k.dx);
  }
  const int band = (nr - wd) * nz;  // first outer row
  // output pointers in registers (a store through a pointer read from the
  // case record would force the record to be re-read after it)
  float* const whi = static_cast<float*>(k.omega_hi);
  float* const wlo = static_cast<float*>(k.omega_lo);
  auto wval = [&](int c) -> double { return (double)w[c]; };
  // stores the tapered value v (double), rounded to T
  auto put = [&](int c, double v) {
    const T h = (T)v;
    w[c] = h;
    if constexpr (sizeof(T) == 4) {
      if (whi) {
        float hi, lo;
        axi_tc::tf32_split((float)h, hi, lo);
        whi[c] = hi;
        wlo[c] = lo;
      }
    }
  };
  // edge columns 0 .. w - 1 and nz - w .. nz - 1 of the outer rows (block 0):
  // the z-tapered value of row nr - w, rounded to T as the reference stores it
  const int t = threadIdx.x;
  const bool edge = blockIdx.x == 0 && t < 2 * wd;
  const int je = t < wd ? t : nz - 2 * wd + t;
  double esrc = 0.0;
  if (edge)
    esrc = (double)(T)(t < wd ? cz0[t] * wval(band + wd - 1) : cz1[t - wd] * wval(band + nz - wd));
  __syncthreads();
  if (edge) {
    for (int q = 0; q < wd; ++q) put(band + q * nz + je, cr[q] * esrc);
    put(je, 0.0);
  }
  const int n_units = nz + (nr - wd - 1 > 0 ? nr - wd - 1 : 0);
  for (int u = 2 * wd + blockIdx.x * blockDim.x + t; u < n_units; u += gridDim.x * blockDim.x) {
    if (u < nz) {
      const int j = u - wd;  // inner column w .. nz - w - 1
      const double src = wval(band + j);
      for (int q = 0; q < wd; ++q) put(band + q * nz + j, cr[q] * src);
      put(j, 0.0);
    } else {
      const int row = (1 + u - nz) * nz;  // rows 1 .. nr - w - 1
      const double left = wval(row + wd - 1);
      const double right = wval(row + nz - wd);
      for (int q = 0; q < wd; ++q) put(row + q, cz0[q] * left);
      for (int q = 0; q < wd; ++q) put(row + nz - wd + q, cz1[q] * right);
    }
  }
}

// ---------------------------------------------------------------------------
// velocity from psi (kernels/compute_velocity_from_psi.py:9-17) plus the free
// stream. psi(a, b) is an accessor; rinv = 1 / (2 dx r_i). The one-sided rows
// and columns at the grid edges (the r = 0 axis closure, the outer r row and
// the z ends): in the double engine the reference's expression in double; in
// the float engine the three-point difference of the float psi values is
// formed with one rounding (edge_diff_exact: what double arithmetic gives for
// these inputs), since it cancels most of its terms at the axis, where
// psi ~ r^2.
// ---------------------------------------------------------------------------
using axi_eft::pair_add;
using axi_eft::two_prod;
using axi_eft::two_sum;

// -p2 + 4 p1 - 3 p0 of float values with a single final rounding (the value
// FP64 arithmetic gives for these float inputs, rounded to float): the
// one-sided difference of the axis closure and the other grid edges cancels
// most of its terms where psi ~ r^2.
__device__ __forceinline__ float edge_diff_exact(float p2, float p1, float p0) {
  float b, be, s1, e1, s2, e2;
  two_prod(3.0f, p0, b, be);
  two_sum(4.0f * p1, -b, s1, e1);
  two_sum(s1, -p2, s2, e2);
  return __fadd_rn(s2, __fsub_rn(__fadd_rn(e1, e2), be));
}

// With a low-part accessor `lo` (float engine, psi carried as psi + psi_lo)
// every difference is the difference of the high parts plus that of the low
// parts.
struct NoLow {
  __device__ float operator()(int, int) const { return 0.0f; }
};

template <typename T, typename Acc, typename Lo = NoLow>
__device__ __forceinline__ void velocity_at(const axi_case& k, Acc psi, int i, int j, T rinv,
                                            T ufree, T& uz, T& ur, Lo lo = Lo()) {
  constexpr bool PAIR = !std::is_same<Lo, NoLow>::value;
  const int nr = k.nr, nz = k.nz;
  if (i == 0 || i == nr - 1) {
    if constexpr (sizeof(T) == 8) {
      double d;
      if (i == 0)
        d = -(double)psi(2, j) + 4.0 * (double)psi(1, j) - 3.0 * (double)psi(0, j);
      else
        d = (double)psi(nr - 3, j) - 4.0 * (double)psi(nr - 2, j) + 3.0 * (double)psi(nr - 1, j);
      uz = (T)(d * (0.5 / k.dx) / k.r[i]) + ufree;
    } else {
      T d = i == 0 ? edge_diff_exact(psi(2, j), psi(1, j), psi(0, j))
                   : -edge_diff_exact(psi(nr - 3, j), psi(nr - 2, j), psi(nr - 1, j));
      if constexpr (PAIR)
        d += i == 0 ? -lo(2, j) + T(4) * lo(1, j) - T(3) * lo(0, j)
                    : lo(nr - 3, j) - T(4) * lo(nr - 2, j) + T(3) * lo(nr - 1, j);
      uz = d * rinv + ufree;
    }
  } else {
    T d = psi(i + 1, j) - psi(i - 1, j);
    if constexpr (PAIR) d += lo(i + 1, j) - lo(i - 1, j);
    uz = d * rinv + ufree;
  }
  if (j == 0 || j == nz - 1) {
    if constexpr (sizeof(T) == 8) {
      double d;
      if (j == 0)
        d = -(double)psi(i, 2) + 4.0 * (double)psi(i, 1) - 3.0 * (double)psi(i, 0);
      else
        d = (double)psi(i, nz - 3) - 4.0 * (double)psi(i, nz - 2) + 3.0 * (double)psi(i, nz - 1);
      ur = (T)(-d) * rinv;
    } else {
      T d = j == 0 ? edge_diff_exact(psi(i, 2), psi(i, 1), psi(i, 0))
                   : -edge_diff_exact(psi(i, nz - 3), psi(i, nz - 2), psi(i, nz - 1));
      if constexpr (PAIR)
        d += j == 0 ? -lo(i, 2) + T(4) * lo(i, 1) - T(3) * lo(i, 0)
                    : lo(i, nz - 3) - T(4) * lo(i, nz - 2) + T(3) * lo(i, nz - 1);
      ur = -d * rinv;
    }
  } else {
    T d = psi(i, j + 1) - psi(i, j - 1);
    if constexpr (PAIR) d += lo(i, j + 1) - lo(i, j - 1);
    ur = -d * rinv;
  }
}

// ---------------------------------------------------------------------------
// Persistent stencil kernels. Each block walks the tile table with stride
// gridDim.x. Thread 0 keeps a ring of NBUF shared-memory box sets: the boxes
// of the tile NBUF - 1 iterations ahead are requested by TMA
// (cp.async.bulk.tensor.2d, zero fill outside the grid) while the current
// tile is computed, so global latency overlaps the arithmetic. Every box is
// BOXW = TX + 8 columns wide starting at column j0 - 4 (a 16-byte aligned
// origin) and HALO rows above the tile. The per-case reductions keep the
// "last tile of the case finalises" pattern: only thread 0 acts on it, so the
// block moves on to its next tile without waiting for the atomics.
// ---------------------------------------------------------------------------
constexpr int BOXW = TX + 8;
constexpr int PSI_ROWS = TY + 4;  // psi and chi boxes: rows i0 - 2 .. i0 + TY + 1
constexpr int ADV_ROWS = TY + 8;  // omega, u_z, u_r boxes: rows i0 - 4 .. i0 + TY + 3
// vel_max is light on arithmetic and runs persistent with a 3-deep ring;
// penalise and advect_diffuse are bound by instruction issue, so they run one
// tile per block (ring depth 1) to keep more blocks resident per SM.
constexpr int VM_NBUF = 3, PN_NBUF = 1, AD_NBUF = 1;

// Ring of box sets in dynamic shared memory (128-byte aligned) and its
// mbarriers (one per slot, one arrival + the boxes' bytes).
template <typename T, int NBUF, int NBOX, int ROWS>
struct BoxRing {
  static constexpr int BOX = ROWS * BOXW;                   // elements per box
  static constexpr uint32_t SET_BYTES = NBOX * BOX * sizeof(T);
  static constexpr int BYTES = NBUF * (int)SET_BYTES;
  T* base;
  uint32_t bar0;
  __device__ T* box(int slot, int which) const { return base + (slot * NBOX + which) * BOX; }
  __device__ void init() const {
    for (int b = 0; b < NBUF; ++b) axi_tma::mbar_init(bar0 + 8 * b, 1);
    axi_tma::fence_mbar_init();
  }
  // thread 0: request the boxes of tile tr into slot `slot`
  __device__ void issue(const CUtensorMap* maps, const int4& tr, const int (&which)[NBOX],
                        int row0, int slot) const {
    const uint32_t bar = bar0 + 8 * slot;
    axi_tma::fence_proxy_async_smem();
    axi_tma::mbar_expect_tx(bar, SET_BYTES);
    for (int q = 0; q < NBOX; ++q)
      axi_tma::tma_load_2d(axi_tma::smem_u32(box(slot, q)), maps + MAP_COUNT * tr.x + which[q],
                           tr.z - 4, tr.y + row0, bar);
  }
  // thread 0: ask L2 for the boxes of tile tr (a hint: no shared memory, no
  // barrier; the box origin clamped into the grid)
  __device__ void prefetch(const CUtensorMap* maps, const int4& tr, const int (&which)[NBOX],
                           int row0) const {
    for (int q = 0; q < NBOX; ++q)
      axi_tma::tma_prefetch_2d(maps + MAP_COUNT * tr.x + which[q], max(tr.z - 4, 0),
                               max(tr.y + row0, 0));
  }
  // Block-wide: thread 0 waits (bounded) for the boxes of iteration `it`,
  // the other threads wait at the barrier (no issue slots spent polling);
  // false on failure, for every thread.
  __device__ bool wait_all(int it, int* err) const {
    int failed = 0;
    if (threadIdx.x == 0)
      failed = !axi_tma::mbar_wait(bar0 + 8 * (it % NBUF), (it / NBUF) & 1, err,
                                   ERR_STENCIL_WAIT);
    return !__syncthreads_or(failed);
  }
  // thread 0, after a failure: wait (bounded) for the copies still in flight
  __device__ void drain(int consumed, int issued, int* err) const {
    for (int g = consumed; g < issued; ++g)
      if (!axi_tma::mbar_wait_drain(bar0 + 8 * (g % NBUF), (g / NBUF) & 1))
        atomicCAS(err, 0, ERR_STENCIL_DRAIN);
  }
};

__device__ __forceinline__ unsigned char* align_smem(unsigned char* p) {
  return reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(p) + 127) &
                                          ~static_cast<uintptr_t>(127));
}

// Issues the prologue of a block's ring; returns how many tiles were issued.
template <typename Ring, int NBUF, int NBOX>
__device__ __forceinline__ int ring_prologue(const Ring& ring, const CUtensorMap* maps,
                                             const int4* tiles, int n_tiles,
                                             const int (&which)[NBOX], int row0) {
  int issued = 0;
  for (int b = 0; b < NBUF - 1; ++b) {
    const int t = blockIdx.x + b * gridDim.x;
    if (t < n_tiles) {
      ring.issue(maps, tiles[t], which, row0, b);
      ++issued;
    }
  }
  return issued;
}

// ---------------------------------------------------------------------------
// vel_max: max over the case of |u_z| + |u_r| (flow_past_sphere.py:150-153),
// atomic maxima per warp; the last block to finish (a grid-wide arrival
// count, reset by kill_reset each step) turns every case's maximum into dt,
// so no tile waits on another.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ unsigned long long order_bits(T v) {
  // non-negative values order like their bit patterns; a NaN sorts above +inf
  return sizeof(T) == 8 ? (unsigned long long)__double_as_longlong((double)v)
                        : (unsigned long long)__float_as_uint((float)v);
}

// dt = min(diffusive limit, CFL / max(|u_z| + |u_r|)) (flow_past_sphere.py:150-155)
// from the maximum that vel_max left in the state block. Every block that
// needs dt evaluates it from the same bits, so all get the same value.
template <typename T>
__device__ __forceinline__ double step_dt(const axi_case& k, double* umax_out = nullptr) {
  const unsigned long long mb =
      *reinterpret_cast<const volatile unsigned long long*>(&k.state[AXI_ST_UMAX]);
  const double umax = sizeof(T) == 8 ? __longlong_as_double((long long)mb)
                                     : (double)__uint_as_float((unsigned int)mb);
  if (umax_out) *umax_out = umax;
  return fmin(k.dt_diff, (k.cfl * k.dx) / (umax + k.eps));
}

// dt and the dt-dependent constants of the step for one case (double state
// words and the float copies), once vel_max has its maximum.
template <typename T>
__device__ __forceinline__ void finish_step_dt(const axi_case& k) {
  double umax;
  const double dt = step_dt<T>(k, &umax);
  if (!(umax <= 1.7976931348623157e308))
    atomicOr(reinterpret_cast<unsigned int*>(&k.state[AXI_ST_STATUS]), 1u << AXI_ERR_NONFINITE);
  k.state[AXI_ST_DT] = dt;
  k.state[AXI_ST_LAMDT] = k.lam * dt;
  k.state[AXI_ST_ADV] = -dt / k.dx;
  k.state[AXI_ST_C1] = 0.5 * k.nu * dt;
  k.state[AXI_ST_C2] = k.nu * dt;
  float* f = fslots(k);
  f[SF_LAMDT] = (float)(k.lam * dt);
  f[SF_ADV] = (float)(-dt / k.dx);
  f[SF_C1] = (float)(0.5 * k.nu * dt);
  f[SF_C2] = (float)(k.nu * dt);
}

// dt comes from the velocities of psi alone, also in the refined float
// engine (the float rounding of psi moves the maximum, and dt, by about 1e-7;
// on the 2000-step FP32-vs-FP64 comparison reading psi_lo here made no
// measurable difference)
template <typename T>
using VmRing = BoxRing<T, VM_NBUF, 1, PSI_ROWS>;
template <typename T>
constexpr int vel_max_smem() {
  return VmRing<T>::BYTES + 128;
}

template <typename T>
__global__ void __launch_bounds__(NT) vel_max_kernel(const axi_case* __restrict__ cases,
                                                     const int4* __restrict__ tiles, int n_tiles,
                                                     const CUtensorMap* __restrict__ maps,
                                                     int* __restrict__ err, int n_cases,
                                                     unsigned int* __restrict__ done) {
  extern __shared__ unsigned char vm_raw[];
  __shared__ __align__(8) uint64_t bars[VM_NBUF];
  VmRing<T> ring{reinterpret_cast<T*>(align_smem(vm_raw)), axi_tma::smem_u32(bars)};
  constexpr int which[1] = {MAP_PSI};
  int issued = 0;
  if (threadIdx.x == 0) {
    ring.init();
    issued = ring_prologue<VmRing<T>, VM_NBUF, 1>(ring, maps, tiles, n_tiles, which, -2);
  }
  __syncthreads();
  // this thread: column tx, rows ty * CPT .. ty * CPT + CPT - 1 of the tile
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  int it = 0;
  bool ok = true;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++it) {
    const int4 tr = tiles[t];
    const axi_case& k = cases[tr.x];
    const int nr = k.nr, nz = k.nz;
    const T* __restrict__ rinv2dx = CF<T>(k.rinv2dx);
    const T ufree = scalar<T>(k, SF_UFREE);
    if (!ring.wait_all(it, err)) {
      ok = false;
      break;
    }
    // past the ring's block barrier every warp has finished tile it - 1, so
    // its slot can take the tile VM_NBUF - 1 ahead
    if (threadIdx.x == 0) {
      const int tn = t + (VM_NBUF - 1) * gridDim.x;
      if (tn < n_tiles) {
        ring.issue(maps, tiles[tn], which, -2, (it + VM_NBUF - 1) % VM_NBUF);
        ++issued;
      }
    }
    const T* bx = ring.box(it % VM_NBUF, 0);
    const int i0 = tr.y, j0 = tr.z;
    auto bp = [&](int gi, int gj) { return bx[(gi - i0 + 2) * BOXW + (gj - j0 + 4)]; };
    const int j = j0 + tx;
    const int ib = i0 + ty * CPT;
    unsigned long long bits = 0;
    if (j < nz) {
      // psi of the rows above and below carried down the column
      T pm = bp(ib - 1, j), pc = bp(ib, j);
#pragma unroll
      for (int m = 0; m < CPT; ++m) {
        const int i = ib + m;
        const T pn = bp(i + 1, j);
        if (i < nr) {
          const T rv = rinv2dx[i];
          T uz, ur;
          if (i == 0 || i == nr - 1 || j == 0 || j == nz - 1) {
            velocity_at<T>(k, bp, i, j, rv, ufree, uz, ur);
          } else {
            uz = (pn - pm) * rv + ufree;
            ur = -(bp(i, j + 1) - bp(i, j - 1)) * rv;
          }
          const unsigned long long b = order_bits<T>(fabs(uz) + fabs(ur));
          bits = b > bits ? b : bits;
        }
        pm = pc;
        pc = pn;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long other = __shfl_down_sync(0xffffffffu, bits, o);
      bits = other > bits ? other : bits;
    }
    // one fire-and-forget atomic maximum per warp (no block barrier: the ring
    // wait at the top of the next tile orders the box reuse); the maximum is
    // read once every block has arrived
    if ((threadIdx.x & 31) == 0 && bits != 0)
      atomicMax(reinterpret_cast<unsigned long long*>(&k.state[AXI_ST_UMAX]), bits);
  }
  if (!ok && threadIdx.x == 0) ring.drain(it, issued, err);
  // every block arrives (a failed one too); the last one sees every tile's
  // atomic maximum and computes dt for all cases
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    for (int c = threadIdx.x; c < n_cases; c += NT) finish_step_dt<T>(cases[c]);
  }
}

// ---------------------------------------------------------------------------
// penalise: flow_past_sphere.py:156-175 (kernels/brinkmann_penalize.py:11-16,
// kernels/compute_vorticity_from_velocity.py:11-13 on u_pen - u, drag).
// Velocity, penalised velocity and their difference are evaluated once per
// point of the tile + halo 1 (owned points also store u_pen and add to the
// drag integrand); the curl of the difference then updates omega of the
// owned cells.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void penalise_point(T uz, T ur, T lc, T ubody, T& pz, T& pr) {
  const T inv = T(1) / (T(1) + lc);
  pz = (uz + lc * ubody) * inv;
  pr = ur * inv;
}

constexpr int PN_SW = TX + 2, PN_SH = TY + 2;  // u_pen - u, halo 1
constexpr int PN_RB = (TY + 2 + RG - 1) / RG;  // rows per group of the halo-1 march
// boxes: psi, chi and, with PAIR (refined float engine), psi_lo
template <typename T, bool PAIR>
using PnRing = BoxRing<T, PN_NBUF, PAIR ? 3 : 2, PSI_ROWS>;
template <typename T, bool PAIR>
constexpr int penalise_smem() {
  return PnRing<T, PAIR>::BYTES + 2 * PN_SH * PN_SW * (int)sizeof(T) + 128;
}
template <typename T, bool PAIR>
constexpr int penalise_min_blocks() {
  return sizeof(T) == 8 ? 2 : (PAIR ? 4 : 5);
}

template <typename T, bool PAIR>
__global__ void __launch_bounds__(NT, penalise_min_blocks<T, PAIR>()) penalise_kernel(
    const axi_case* __restrict__ cases, const int4* __restrict__ tiles, int n_tiles,
    const CUtensorMap* __restrict__ maps, int* __restrict__ err, int ahead) {
  static_assert(!PAIR || sizeof(T) == 4, "psi pairs belong to the float engine");
  constexpr int NB = PAIR ? 3 : 2;
  using Ring = PnRing<T, PAIR>;
  extern __shared__ unsigned char pn_raw[];
  __shared__ __align__(8) uint64_t bars[PN_NBUF];
  __shared__ double red[2][NT / 32];
  __shared__ T rowf[2][PN_SH];  // 1 / (2 dx r), r
  Ring ring{reinterpret_cast<T*>(align_smem(pn_raw)), axi_tma::smem_u32(bars)};
  T* duz = ring.base + Ring::BYTES / sizeof(T);
  T* dur = duz + PN_SH * PN_SW;
  constexpr int which3[3] = {MAP_PSI, MAP_CHI, MAP_PSI_LO};
  const int(&which)[NB] = *reinterpret_cast<const int(*)[NB]>(&which3);
  int issued = 0;
  if (threadIdx.x == 0) {
    ring.init();
    issued = ring_prologue<Ring, PN_NBUF, NB>(ring, maps, tiles, n_tiles, which, -2);
  }
  __syncthreads();
  int it = 0;
  bool ok = true;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++it) {
    if (threadIdx.x == 0) {
      const int tn = t + (PN_NBUF - 1) * gridDim.x;
      if (tn < n_tiles) {
        ring.issue(maps, tiles[tn], which, -2, (it + PN_NBUF - 1) % PN_NBUF);
        ++issued;
      }
      // the tile one resident wave ahead: its boxes wait in L2
      if (t + ahead < n_tiles) ring.prefetch(maps, tiles[t + ahead], which, -2);
    }
    const int4 tr = tiles[t];
    const axi_case& k = cases[tr.x];
    const int nr = k.nr, nz = k.nz;
    const int i0 = tr.y, j0 = tr.z;
    const T* __restrict__ rinv2dx = CF<T>(k.rinv2dx);
    const T* __restrict__ rw = CF<T>(k.rw);
    const T ufree = scalar<T>(k, SF_UFREE);
    const T ubody = scalar<T>(k, SF_UBODY);
    // low part of the body velocity (float engine: U = ubody + ubody_lo)
    T ubody_lo = T(0);
    if constexpr (sizeof(T) == 4) ubody_lo = scalar<T>(k, SF_UBODY_LO);
    const T inv2dx = scalar<T>(k, SF_INV2DX);
    const T* w = CF<T>(k.omega);
    // the penalised vorticity goes to the first nr x nz elements of the work
    // buffer (free between the spectral solve and the next step's solve):
    // advect_diffuse reads its halo rows from there while it writes omega, so
    // no tile reads a neighbour's already-advanced rows
    T* const ws = F<T>(k.gemm_work);
    const T lamdt = scalar<T>(k, SF_LAMDT);
    // per-row factors of the tile + halo 1 (rows i0 - 1 .. i0 + TY)
    if (threadIdx.x < PN_SH) {
      const int gi = min(max(i0 - 1 + (int)threadIdx.x, 0), nr - 1);
      rowf[0][threadIdx.x] = rinv2dx[gi];
      rowf[1][threadIdx.x] = rw[gi];
    }
    if (!ring.wait_all(it, err)) {
      ok = false;
      break;
    }
    const T* ps = ring.box(it % PN_NBUF, 0);
    const T* sc = ring.box(it % PN_NBUF, 1);
    // low part of psi (PAIR); the psi box itself otherwise (never read)
    const T* pl = ring.box(it % PN_NBUF, NB - 1);
    // every one-sided stencil of an edge cell stays inside the box
    auto sp = [&](int gi, int gj) { return ps[(gi - i0 + 2) * BOXW + (gj - j0 + 4)]; };
    auto spl = [&](int gi, int gj) { return pl[(gi - i0 + 2) * BOXW + (gj - j0 + 4)]; };
    T* uzp = F<T>(k.u_z);
    T* urp = F<T>(k.u_r);
    // drag integrand sum of this thread (the float engine forms u_pen - U as
    // (u_z - U) / (1 + lam dt chi), the same value without its cancellation;
    // the sum over the body is well conditioned, sum |t| / |sum t| below 5
    // on the sedimenting cases, so float partial sums suffice)
    T cd_part = T(0);
    // Column march (as in advect_diffuse): warp w owns tile columns
    // 32 (w % 2) .. + 31 and a run of consecutive rows from (w / 2) x rows
    // per group; psi of the rows above and below stays in registers. The
    // psi and chi boxes share one layout: point (p, q) of the tile is
    // element (p + 2) * BOXW + q + 4 of both.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int qm = (warp & 1) * 32 + lane, grp = warp >> 1;
    const int gjm = j0 + qm;
    // u_pen - u at one point of the tile + halo 1 (p in [-1, TY], q in [-1, TX])
    auto point = [&](int p, int q, T uz, T ur, T ch, int gi, int gj) {
      T pz, pr, dz, dr;
      if constexpr (sizeof(T) == 8) {
        penalise_point<T>(uz, ur, lamdt * ch, ubody, pz, pr);
        dz = pz - uz;
        dr = pr - ur;
      } else {
        // u_pen - u = lam dt chi (U - u) / (1 + lam dt chi), formed directly:
        // inside the body u is close to U, and the difference of the rounded
        // u_pen and u would keep only the rounding of u_pen (its curl, / dx,
        // is vorticity noise of ulp(U) / dx per step); U = ubody + ubody_lo
        const T lc = lamdt * ch;
        const T inv = T(1) / (T(1) + lc);
        const T du = (ubody - uz) + ubody_lo;
        dz = (lc * inv) * du;
        dr = -(lc * inv) * ur;
        pz = uz + dz;
        pr = ur + dr;
        if (p >= 0 && p < TY && q >= 0 && q < TX)
          cd_part -= rowf[1][p + 1] * ch * (du * inv);
      }
      const int d = (p + 1) * PN_SW + (q + 1);
      duz[d] = dz;
      dur[d] = dr;
      if (p >= 0 && p < TY && q >= 0 && q < TX) {
        const int c = gi * nz + gj;
        uzp[c] = pz;
        urp[c] = pr;
        // drag / penalisation force integrand r chi (u_z - U_body)
        // (flow_past_sphere.py:173, compute_forces.py:14); the float engine
        // adds it above as -r chi (U - u) / (1 + lam dt chi)
        if constexpr (sizeof(T) == 8) cd_part += rowf[1][p + 1] * ch * (pz - ubody);
      }
    };
    {
      const bool jin = gjm < nz, jint = gjm >= 1 && gjm < nz - 1;
      const int p0 = -1 + PN_RB * grp;
      int cb = (p0 + 2) * BOXW + (qm + 4);
      T pm = ps[cb - BOXW], pc = ps[cb];
      T lm = T(0), lc = T(0);
      if constexpr (PAIR) {
        lm = pl[cb - BOXW];
        lc = pl[cb];
      }
#pragma unroll
      for (int m = 0; m < PN_RB; ++m, cb += BOXW) {
        const int pr_ = p0 + m;
        if (pr_ > TY) break;
        const T pn = ps[cb + BOXW];
        T ln = T(0);
        if constexpr (PAIR) ln = pl[cb + BOXW];
        const int gi = i0 + pr_;
        if (jin && gi >= 0 && gi < nr) {
          const T rv = rowf[0][pr_ + 1];
          const T ch = sc[cb];
          T uz, ur;
          if (gi == 0 || gi == nr - 1 || !jint) {
            if constexpr (PAIR)
              velocity_at<T>(k, sp, gi, gjm, rv, ufree, uz, ur, spl);
            else
              velocity_at<T>(k, sp, gi, gjm, rv, ufree, uz, ur);
          } else if constexpr (PAIR) {
            uz = ((pn - pm) + (ln - lm)) * rv + ufree;
            ur = -((ps[cb + 1] - ps[cb - 1]) + (pl[cb + 1] - pl[cb - 1])) * rv;
          } else {
            uz = (pn - pm) * rv + ufree;
            ur = -(ps[cb + 1] - ps[cb - 1]) * rv;
          }
          point(pr_, qm, uz, ur, ch, gi, gjm);
        } else {
          const int d = (pr_ + 1) * PN_SW + (qm + 1);
          duz[d] = T(0);
          dur[d] = T(0);
        }
        pm = pc;
        pc = pn;
        lm = lc;
        lc = ln;
      }
      // halo columns -1 and TX
      if (threadIdx.x < 2 * PN_SH) {
        const int pe = -1 + (int)threadIdx.x / 2, qe = (threadIdx.x & 1) ? TX : -1;
        const int gi = i0 + pe, gj = j0 + qe;
        if (gi >= 0 && gi < nr && gj >= 0 && gj < nz) {
          T uz, ur;
          if constexpr (PAIR)
            velocity_at<T>(k, sp, gi, gj, rowf[0][pe + 1], ufree, uz, ur, spl);
          else
            velocity_at<T>(k, sp, gi, gj, rowf[0][pe + 1], ufree, uz, ur);
          point(pe, qe, uz, ur, sc[(pe + 2) * BOXW + (qe + 4)], gi, gj);
        } else {
          const int d = (pe + 1) * PN_SW + (qe + 1);
          duz[d] = T(0);
          dur[d] = T(0);
        }
      }
    }
    // omega of the owned cells (column march, rows 8 grp .. 8 grp + 7):
    // all loads issued before the first use
    constexpr int RC = TY / RG;
    const int p0c = RC * grp;
    T wown[RC];
#pragma unroll
    for (int m = 0; m < RC; ++m) {
      const int gi = i0 + p0c + m;
      wown[m] = (gi < nr && gjm < nz) ? w[gi * nz + gjm] : T(0);
    }
    __syncthreads();
    {
      const bool jin = gjm < nz, jint = gjm >= 1 && gjm < nz - 1;
      int d = (p0c + 1) * PN_SW + (qm + 1);
      T zs = duz[d - PN_SW], zc = duz[d];
#pragma unroll
      for (int m = 0; m < RC; ++m, d += PN_SW) {
        const T zn = duz[d + PN_SW];
        const int gi = i0 + p0c + m;
        if (jin && gi < nr) {
          T v = wown[m];
          if (jint && gi >= 1 && gi < nr - 1) {
            const T pw = (dur[d + 1] - dur[d - 1]) * inv2dx - (zn - zs) * inv2dx;
            v = wown[m] + pw;
          }
          ws[gi * nz + gjm] = v;
        }
        zs = zc;
        zc = zn;
      }
    }
    // drag: thread sums in T, then warps, tiles and cases in double, fixed order
    double x = cd_part;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[it & 1][threadIdx.x >> 5] = (double)x;
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned int ntiles = dev_tiles_of(k);
      double sum = 0.0;
      for (int q = 0; q < NT / 32; ++q) sum += red[it & 1][q];
      k.partials[tr.w] = sum;
      __threadfence();
      if (atomicAdd(counter(k, 1), 1u) == ntiles - 1) {
        __threadfence();
        double tot = 0.0;
        for (unsigned int q = 0; q < ntiles; ++q) tot += ((volatile double*)k.partials)[q];
        const double dt = k.state[AXI_ST_DT];
        if (!(tot == tot) || !(fabs(tot) <= 1.7976931348623157e308))
          atomicOr(reinterpret_cast<unsigned int*>(&k.state[AXI_ST_STATUS]),
                   1u << AXI_ERR_NONFINITE);
        k.state[AXI_ST_FORCE] = tot;
        if (k.flags & AXI_CASE_SEDIMENTING) {
          // compute_forces.py:14-15 and falling_rigid_sphere.py:155
          const double f_pen = k.rho_f * k.lam * tot;
          const double f_un = (k.state[AXI_ST_DIFF] * k.part_vol) / dt;
          k.state[AXI_ST_FTOTAL] = 2.0 * kPi * k.dx * k.dx * f_pen + f_un;
        } else {
          const double cd = k.cd_scale * tot;
          const long long step = (long long)k.state[AXI_ST_STEPS];
          if (k.history && step < k.history_len) {
            k.history[2 * step] = dt;
            k.history[2 * step + 1] = cd;
          }
          k.state[AXI_ST_CD] = cd;
        }
      }
    }
  }
  if (!ok && threadIdx.x == 0) ring.drain(it, issued, err);
}

// ---------------------------------------------------------------------------
// ENO3 face flux (pyst_kernels/advection_flux.py:9-163)
// ---------------------------------------------------------------------------
// FP32 engine: the face flux from the flux values g = f u of the four points
// (formed once, shared by both upwind branches and by neighbouring faces)
template <typename T>
__device__ __forceinline__ T face_flux_g(T gm1, T g0, T g1, T g2, T u0, T u1) {
  const T third = T(1) / T(3), five6 = T(5) / T(6), sixth = T(1) / T(6);
  const T a = third * g1 + five6 * g0 - sixth * gm1;
  const T b = third * g0 + five6 * g1 - sixth * g2;
  return u0 > -u1 ? a : b;
}

template <typename T>
__device__ __forceinline__ T face_flux(T fm1, T f0, T f1, T f2, T um1, T u0, T u1, T u2) {
  const T third = T(1) / T(3), five6 = T(5) / T(6), sixth = T(1) / T(6);
  if constexpr (sizeof(T) == 4) {
    return face_flux_g(fm1 * um1, f0 * u0, f1 * u1, f2 * u2, u0, u1);
  } else {
    // the reference's products and order (bit-exact with the FP64 oracle)
    if (u0 > -u1) return third * f1 * u1 + five6 * f0 * u0 - sixth * fm1 * um1;
    return third * f0 * u0 + five6 * f1 * u1 - sixth * f2 * u2;
  }
}

// FP32 engine: the ENO3 flux divergence F(i+1/2) - F(i-1/2) of one direction
// formed from differences of neighbouring flux values instead of the two face
// values. Each face value is its upwind cell's flux value g = f u plus a
// small correction, (1/3)(g1 - g0) - (1/6)(gm1 - g0) for the branch u0 > -u1
// and (1/3)(g0 - g1) - (1/6)(g2 - g1) otherwise (the same weights 1/3, 5/6,
// -1/6), so the divergence is a combination of the four differences
// d_k = g(k+1) - g(k) around the cell. With g an exact product pair and each
// difference taken pairwise, the rounding of the result scales with the
// differences, not with |g|: the face values of a smooth field no longer
// cancel in float.
struct GPair {
  float h, l;
};
__device__ __forceinline__ GPair gprod(float f, float u) {
  GPair g;
  g.h = __fmul_rn(f, u);
  g.l = fmaf(f, u, -g.h);
  return g;
}
// g(b) - g(a)
__device__ __forceinline__ float gdiff(GPair a, GPair b) {
  return __fadd_rn(__fsub_rn(b.h, a.h), __fsub_rn(b.l, a.l));
}
// d0 = g(i-1) - g(i-2), d1 = g(i) - g(i-1), d2 = g(i+1) - g(i), d3 = g(i+2) - g(i+1);
// af, ab: the upwind tests of the faces i+1/2 (u_i > -u_{i+1}) and i-1/2
__device__ __forceinline__ float eno3_div(float d0, float d1, float d2, float d3, bool af,
                                          bool ab) {
  const float third = 1.0f / 3.0f, sixth = 1.0f / 6.0f;
  const float cf = af ? fmaf(third, d2, __fmul_rn(sixth, d1))
                      : -fmaf(third, d2, __fmul_rn(sixth, d3));
  const float cb = ab ? fmaf(third, d1, __fmul_rn(sixth, d0))
                      : -fmaf(third, d1, __fmul_rn(sixth, d2));
  // upwind cells of the two faces: (i, i-1) -> d1, (i, i) -> 0,
  // (i+1, i-1) -> d1 + d2, (i+1, i) -> d2
  const float base = af ? (ab ? d1 : 0.0f) : (ab ? __fadd_rn(d1, d2) : d2);
  return __fsub_rn(__fadd_rn(base, cf), cb);
}
// divergence along a line of five values f, u at stride `st` around c
__device__ __forceinline__ float eno3_div_at(const float* f, const float* u, int c, int st) {
  const GPair gm2 = gprod(f[c - 2 * st], u[c - 2 * st]), gm1 = gprod(f[c - st], u[c - st]);
  const GPair g0 = gprod(f[c], u[c]), g1 = gprod(f[c + st], u[c + st]);
  const GPair g2 = gprod(f[c + 2 * st], u[c + 2 * st]);
  return eno3_div(gdiff(gm2, gm1), gdiff(gm1, g0), gdiff(g0, g1), gdiff(g1, g2),
                  u[c] > -u[c + st], u[c - st] > -u[c]);
}
// the advected value f0 + a (Dx + Dy)
__device__ __forceinline__ float eno3_update(float f0, float a, float dxv, float dyv) {
  return __fadd_rn(f0, __fadd_rn(__fmul_rn(a, dxv), __fmul_rn(a, dyv)));
}

// RK2 operator at one cell (kernels/diffusion_RK2.py:15-25). The FP64 engine
// keeps the reference's expression; the FP32 engine sums the four neighbour
// differences (exact for neighbouring values within a factor 2) instead of
// n + s + e + w - 4 c, whose float rounding scales with |c|.
template <typename T>
__device__ __forceinline__ T rk2_lap(T n, T s, T e, T w, T c, T inv_dx2, T k1, T k2) {
  if constexpr (sizeof(T) == 4) {
    const T ns = __fadd_rn(__fsub_rn(n, c), __fsub_rn(s, c));
    const T ew = __fadd_rn(__fsub_rn(e, c), __fsub_rn(w, c));
    return __fmul_rn(__fadd_rn(ns, ew), inv_dx2) + (n - s) * k1 - c * k2;
  } else {
    return (n + s + e + w - T(4) * c) * inv_dx2 + (n - s) * k1 - c * k2;
  }
}

// Smoothed Heaviside of a sphere level set (kernels/smooth_Heaviside.py:10-14,
// level set of falling_rigid_sphere.py:156).
template <typename T>
__device__ __forceinline__ T sphere_mask(T z, T r, T zc, T radius, T w) {
  const T dz = z - zc;
  const T phi = -sqrt(dz * dz + r * r) + radius;
  T h = phi >= w ? T(1) : T(0);
  if (fabs(phi) < w) h += T(0.5) * (T(1) + phi / w + dev_sin(Pi<T>::v * phi / w) / Pi<T>::v);
  return h;
}

// The float engine's moving-body mask, in cell units: t = j + 1/2 - z_cm / dx,
// q = i + 1/2, level set phi = R - sqrt(t^2 + q^2) with R = radius / dx. A
// float estimate decides the cells well inside (1) and outside (0) the blend
// band |phi| < W; within the band (and the estimate's error of it) phi is
// formed as (R^2 - t^2 - q^2) / (R + sqrt(t^2 + q^2)) with the squares and
// the difference carried as exact float pairs, from the hi / lo splits of
// z_cm / dx and R, so the mask follows the double body position (a float
// z_cm alone is off by up to 6e-8 absolute, i.e. 5e-5 of the blend width at
// dx = 1/512, and shifts every band cell the same way).
__device__ __forceinline__ float sphere_mask_cells(int i, int j, float s_hi, float s_lo,
                                                   float r_hi, float r_lo, float w) {
  const float t = __fsub_rn((float)j + 0.5f, s_hi);  // exact near the body
  const float q = (float)i + 0.5f;
  const float q2 = q * q;                            // exact (q <= 2^11)
  const float est = r_hi - sqrtf(fmaf(t, t, q2));
  if (fabsf(est) >= w + 1e-3f) return est >= w ? 1.0f : 0.0f;
  // D = t_true^2 + q^2 with t_true = t - s_lo; R^2 = r_hi^2 + 2 r_hi r_lo
  float a, ae, d_hi, d_e, c, ce, n_hi, n_e;
  two_prod(t, t, a, ae);
  two_sum(a, q2, d_hi, d_e);
  const float d_lo = __fadd_rn(__fadd_rn(d_e, ae), -2.0f * t * s_lo);
  two_prod(r_hi, r_hi, c, ce);
  const float c_lo = __fadd_rn(ce, 2.0f * r_hi * r_lo);
  two_sum(c, -d_hi, n_hi, n_e);
  const float num = __fadd_rn(n_hi, __fsub_rn(__fadd_rn(n_e, c_lo), d_lo));
  const float phi = num / (r_hi + sqrtf(d_hi));
  float h = phi >= w ? 1.0f : 0.0f;
  if (fabsf(phi) < w) h += 0.5f * (1.0f + phi / w + sinf(3.14159265f * phi / w) / 3.14159265f);
  return h;
}

// ---------------------------------------------------------------------------
// advect_diffuse: ENO3 advection (kernels/advect_vorticity_via_eno3.py:28-42,
// pyst_kernels/advection_flux.py:9-163, advection_timestep.py:37-54) followed
// by both RK2 diffusion stages (kernels/diffusion_RK2.py:9-44), fused: the
// boxes of the penalised omega (staged in the work buffer by penalise), u_z
// and u_r (halo 4) arrive by TMA; the block advects the tile plus a halo of
// 2, applies stage 1 on the tile plus a halo of 1 and stage 2 on the tile,
// all in shared memory, and writes omega: each value is read and written once
// per step, and the halo rows a tile reads are never the ones another tile
// has already advanced (blocks of a later wave start after earlier tiles
// were written). Rows below the axis are the mirror images of rows 0..3
// (omega and u_r odd, u_z even). Sedimenting cases also rebuild the body mask
// here and close the step (falling_rigid_sphere.py:156-181).
// ---------------------------------------------------------------------------
constexpr int AD_H = 4;
constexpr int AD_AW = TX + 4, AD_AH = TY + 4;    // advected (halo 2)
constexpr int AD_SW = TX + 2, AD_SH = TY + 2;    // stage 1 (halo 1)
template <typename T>
using AdRing = BoxRing<T, AD_NBUF, 3, ADV_ROWS>;
template <typename T>
constexpr int advect_diffuse_smem() {
  return AdRing<T>::BYTES + (int)sizeof(T) * AD_AH * AD_AW + 128;
}

// Tile-relative indices (row p, column q) into the shared arrays: the staged
// boxes (rows -4..TY+3, columns -4..TX+3), the advected values wa (rows
// -2..TY+1, columns -2..TX+1) and the stage-1 values tp (rows -1..TY,
// columns -1..TX).
__device__ __forceinline__ int ad_box(int p, int q) { return (p + AD_H) * BOXW + (q + AD_H); }
__device__ __forceinline__ int ad_wa(int p, int q) { return (p + 2) * AD_AW + (q + 2); }
__device__ __forceinline__ int ad_tp(int p, int q) { return (p + 1) * AD_SW + (q + 1); }
// rows per thread of the column march: advection (TY + 4 rows), stage 1
// (TY + 2 rows, one spare), stage 2 (TY rows), over RG row groups
constexpr int AD_RA = (TY + 4) / RG, AD_RC = TY / RG;
static_assert(AD_RA * RG == TY + 4 && AD_RA * RG >= TY + 2 && AD_RC * RG == TY, "row groups");
static_assert(2 * 32 == TX && NT == 8 * 32, "two warps per row group");

// Advected omega at one point with all four face fluxes evaluated here (the
// halo columns of the tile).
template <typename T>
__device__ __forceinline__ T advect_point(const T* sw, const T* sz, const T* sr, int p, int q,
                                          int gi, int gj, int nr, int nz, T a) {
  if (!(gi >= 0 && gi < nr && gj >= 0 && gj < nz)) return T(0);
  const int c = ad_box(p, q);
  const T f0 = sw[c];
  if constexpr (sizeof(T) == 4) {
    if (gi < nr - 2 && gj >= 2 && gj < nz - 2)
      return eno3_update(f0, a, eno3_div_at(sw, sz, c, 1), eno3_div_at(sw, sr, c, BOXW));
    return f0;
  }
  T flux = T(0);
  if (gi < nr - 2 && gj >= 2 && gj < nz - 2) {
    const int L = BOXW;
    const T xf = face_flux(sw[c - 1], f0, sw[c + 1], sw[c + 2], sz[c - 1], sz[c], sz[c + 1],
                           sz[c + 2]);
    const T xb = face_flux(sw[c - 2], sw[c - 1], f0, sw[c + 1], sz[c - 2], sz[c - 1], sz[c],
                           sz[c + 1]);
    const T yf = face_flux(sw[c - L], f0, sw[c + L], sw[c + 2 * L], sr[c - L], sr[c], sr[c + L],
                           sr[c + 2 * L]);
    const T yb = face_flux(sw[c - 2 * L], sw[c - L], f0, sw[c + L], sr[c - 2 * L], sr[c - L],
                           sr[c], sr[c + L]);
    flux = a * xf;
    flux = flux - a * xb;
    flux = flux + a * yf;
    flux = flux - a * yb;
  }
  return f0 + flux;
}

// FP32: 4 resident blocks per SM (up to 64 registers; at 5 blocks the
// pairwise flux divergence spilled and ran 5 % slower)
template <typename T>
__global__ void __launch_bounds__(NT, sizeof(T) == 4 ? 4 : 1) advect_diffuse_kernel(const axi_case* __restrict__ cases,
                                                            const int4* __restrict__ tiles,
                                                            int n_tiles,
                                                            const CUtensorMap* __restrict__ maps,
                                                            int* __restrict__ err, int ahead) {
  extern __shared__ unsigned char ad_raw[];
  __shared__ __align__(8) uint64_t bars[AD_NBUF];
  __shared__ double red[2][NT / 32];
  __shared__ T rowf[3][AD_SH];  // 1 / (2 dx r), 1 / r^2, r of rows i0 - 1 .. i0 + TY
  AdRing<T> ring{reinterpret_cast<T*>(align_smem(ad_raw)), axi_tma::smem_u32(bars)};
  T* wa = ring.base + AdRing<T>::BYTES / sizeof(T);
  constexpr int which[3] = {MAP_W, MAP_UZ, MAP_UR};
  int issued = 0;
  if (threadIdx.x == 0) {
    ring.init();
    issued = ring_prologue<AdRing<T>, AD_NBUF, 3>(ring, maps, tiles, n_tiles, which, -AD_H);
  }
  __syncthreads();
  int it = 0;
  bool ok = true;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++it) {
    if (threadIdx.x == 0) {
      const int tn = t + (AD_NBUF - 1) * gridDim.x;
      if (tn < n_tiles) {
        ring.issue(maps, tiles[tn], which, -AD_H, (it + AD_NBUF - 1) % AD_NBUF);
        ++issued;
      }
      // the tile one resident wave ahead: its boxes wait in L2
      if (t + ahead < n_tiles) ring.prefetch(maps, tiles[t + ahead], which, -AD_H);
    }
    const int4 tr = tiles[t];
    const axi_case& k = cases[tr.x];
    const int nr = k.nr, nz = k.nz;
    const int i0 = tr.y, j0 = tr.z;
    const T* __restrict__ rinv2dx = CF<T>(k.rinv2dx);
    const T* __restrict__ rinv2 = CF<T>(k.rinv2);
    const T a = scalar<T>(k, SF_ADV);
    const T c1 = scalar<T>(k, SF_C1);
    const T c2 = scalar<T>(k, SF_C2);
    const T inv_dx2 = scalar<T>(k, SF_INVDX2);
    if (threadIdx.x < AD_SH) {
      const int gi = min(max(i0 - 1 + (int)threadIdx.x, 0), nr - 1);
      rowf[0][threadIdx.x] = rinv2dx[gi];
      rowf[1][threadIdx.x] = rinv2[gi];
      rowf[2][threadIdx.x] = CF<T>(k.rw)[gi];
    }
    if (!ring.wait_all(it, err)) {
      ok = false;
      break;
    }
    T* sw = ring.box(it % AD_NBUF, 0);
    T* sz = ring.box(it % AD_NBUF, 1);
    T* sr = ring.box(it % AD_NBUF, 2);
    // RK2 stage 1 reuses the omega box once the advected values are in wa
    T* tp = sw;
    static_assert(AD_SH * AD_SW <= ADV_ROWS * BOXW, "stage-1 tile fits the omega box");
    if (i0 == 0) {
      // box rows 0..3 (global rows -4..-1) mirror box rows 7..4 (rows 3..0)
      for (int e = threadIdx.x; e < AD_H * BOXW; e += NT) {
        const int p = e / BOXW, q = e - p * BOXW;
        const int gj = j0 - AD_H + q;
        if (gj >= 0 && gj < nz) {
          const int src = (2 * AD_H - 1 - p) * BOXW + q;
          sw[e] = -sw[src];
          sz[e] = sz[src];
          sr[e] = -sr[src];
        }
      }
      __syncthreads();
    }
    // Work split of the three passes: warp w owns tile columns
    // 32 (w % 2) .. 32 (w % 2) + 31 and a run of consecutive rows starting at
    // (w / 2) x (rows per group), so each thread marches down one column and
    // keeps the values of the rows above and below it in registers; the
    // halo columns left and right of the tile are separate small loops.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int qm = (warp & 1) * 32 + lane;  // tile column of the column march
    const int grp = warp >> 1;              // row group 0..3
    const int gjm = j0 + qm;
    constexpr int L = BOXW;
    // ---- advected omega on the tile + halo 2: rows -2..TY+1, columns -2..TX+1
    if constexpr (sizeof(T) == 4) {
      // FP32: the r-direction flux values of the window rows ride along as
      // exact pairs with their differences (one new product and one new
      // difference per row)
      const bool jin = gjm < nz, jflux = gjm >= 2 && gjm < nz - 2;
      const int p0 = -2 + AD_RA * grp;
      int c = ad_box(p0, qm);
      const GPair gm2 = gprod(sw[c - 2 * L], sr[c - 2 * L]);
      const GPair gm1 = gprod(sw[c - L], sr[c - L]);
      const GPair g0 = gprod(sw[c], sr[c]);
      GPair g1 = gprod(sw[c + L], sr[c + L]);
      float d0 = gdiff(gm2, gm1), d1 = gdiff(gm1, g0), d2 = gdiff(g0, g1);
      float f0 = sw[c], f1 = sw[c + L], u0 = sr[c], u1 = sr[c + L];
      bool ab = sr[c - L] > -u0;
#pragma unroll 1
      for (int m = 0; m < AD_RA; ++m, c += L) {
        const int pr = p0 + m, gi = i0 + pr;
        const float f2 = sw[c + 2 * L], u2 = sr[c + 2 * L];
        const GPair g2 = gprod(f2, u2);
        const float d3 = gdiff(g1, g2);
        const bool af = u0 > -u1;
        float val = 0.0f;
        if (jin && gi >= 0 && gi < nr) {
          val = f0;
          // pystencils ghost layers: no flux in the last two rows and the
          // first and last two columns
          if (jflux && gi < nr - 2)
            val = eno3_update(f0, a, eno3_div_at(sw, sz, c, 1), eno3_div(d0, d1, d2, d3, af, ab));
        }
        wa[ad_wa(pr, qm)] = val;
        d0 = d1;
        d1 = d2;
        d2 = d3;
        g1 = g2;
        ab = af;
        f0 = f1;
        f1 = f2;
        u0 = u1;
        u1 = u2;
      }
      // halo columns -2, -1, TX, TX + 1
      if (threadIdx.x < 4 * AD_AH) {
        const int pr = -2 + (int)threadIdx.x / 4, s4 = threadIdx.x % 4;
        const int qe = s4 < 2 ? s4 - 2 : TX + s4 - 2;
        wa[ad_wa(pr, qe)] = advect_point<T>(sw, sz, sr, pr, qe, i0 + pr, j0 + qe, nr, nz, a);
      }
    } else {
      const bool jin = gjm < nz, jflux = gjm >= 2 && gjm < nz - 2;
      const int p0 = -2 + AD_RA * grp;
      int c = ad_box(p0, qm);
      // r-direction face fluxes: yb of row p is yf of row p - 1
      T fm2 = sw[c - 2 * L], fm1 = sw[c - L], f0 = sw[c], f1 = sw[c + L];
      T um2 = sr[c - 2 * L], um1 = sr[c - L], u0 = sr[c], u1 = sr[c + L];
      T yb = face_flux(fm2, fm1, f0, f1, um2, um1, u0, u1);
#pragma unroll 1
      for (int m = 0; m < AD_RA; ++m, c += L) {
        const int pr = p0 + m, gi = i0 + pr;
        const T f2 = sw[c + 2 * L], u2 = sr[c + 2 * L];
        const T yf = face_flux(fm1, f0, f1, f2, um1, u0, u1, u2);
        T val = T(0);
        if (jin && gi >= 0 && gi < nr) {
          T flux = T(0);
          // pystencils ghost layers: no flux in the last two rows and the
          // first and last two columns
          if (jflux && gi < nr - 2) {
            const T xf = face_flux(sw[c - 1], f0, sw[c + 1], sw[c + 2], sz[c - 1], sz[c],
                                   sz[c + 1], sz[c + 2]);
            const T xb = face_flux(sw[c - 2], sw[c - 1], f0, sw[c + 1], sz[c - 2], sz[c - 1],
                                   sz[c], sz[c + 1]);
            flux = a * xf;
            flux = flux - a * xb;
            flux = flux + a * yf;
            flux = flux - a * yb;
          }
          val = f0 + flux;
        }
        wa[ad_wa(pr, qm)] = val;
        yb = yf;
        fm2 = fm1;
        fm1 = f0;
        f0 = f1;
        f1 = f2;
        um2 = um1;
        um1 = u0;
        u0 = u1;
        u1 = u2;
      }
      // halo columns -2, -1, TX, TX + 1
      if (threadIdx.x < 4 * AD_AH) {
        const int pr = -2 + (int)threadIdx.x / 4, s4 = threadIdx.x % 4;
        const int qe = s4 < 2 ? s4 - 2 : TX + s4 - 2;
        wa[ad_wa(pr, qe)] = advect_point<T>(sw, sz, sr, pr, qe, i0 + pr, j0 + qe, nr, nz, a);
      }
    }
    __syncthreads();
    // ---- RK2 stage 1 on the tile + halo 1: rows -1..TY, columns -1..TX
    {
      const bool jin = gjm < nz, jint = gjm >= 1 && gjm < nz - 1;
      const int p0 = -1 + AD_RA * grp;
      int d = ad_wa(p0, qm);
      T s_ = wa[d - AD_AW], c_ = wa[d];
#pragma unroll
      for (int m = 0; m < AD_RA; ++m, d += AD_AW) {
        const int pr = p0 + m;
        if (pr > TY) break;
        const T n_ = wa[d + AD_AW];
        const int gi = i0 + pr;
        T tmpv = T(0);
        if (jin && gi >= 0 && gi < nr) {
          tmpv = c_;
          if (jint && gi >= 1 && gi < nr - 1) {
            const T ee = wa[d + 1], ww = wa[d - 1];
            const T lap = rk2_lap<T>(n_, s_, ee, ww, c_, inv_dx2, rowf[0][pr + 1],
                                     rowf[1][pr + 1]);
            tmpv = c_ + c1 * lap;
          }
        }
        tp[ad_tp(pr, qm)] = tmpv;
        s_ = c_;
        c_ = n_;
      }
      // halo columns -1 and TX
      if (threadIdx.x < 2 * AD_SH) {
        const int pr = -1 + (int)threadIdx.x / 2, qe = (threadIdx.x & 1) ? TX : -1;
        const int gi = i0 + pr, gj = j0 + qe;
        T tmpv = T(0);
        if (gi >= 0 && gi < nr && gj >= 0 && gj < nz) {
          const int e = ad_wa(pr, qe);
          const T c0 = wa[e];
          tmpv = c0;
          if (gi >= 1 && gi < nr - 1 && gj >= 1 && gj < nz - 1) {
            const T n = wa[e + AD_AW], s = wa[e - AD_AW], ee = wa[e + 1], ww = wa[e - 1];
            const T lap = rk2_lap<T>(n, s, ee, ww, c0, inv_dx2, rowf[0][pr + 1],
                                     rowf[1][pr + 1]);
            tmpv = c0 + c1 * lap;
          }
        }
        tp[ad_tp(pr, qe)] = tmpv;
      }
    }
    __syncthreads();
    // ---- RK2 stage 2 on the tile (rows 0..TY-1, columns 0..TX-1)
    const bool sediment = (k.flags & AXI_CASE_SEDIMENTING) != 0;
    T cd_part = T(0);
    {
      // output pointers in registers (stores through pointers read from the
      // case record would force the record to be re-read after each store)
      T* const wout = F<T>(k.omega);
      float* const whi = static_cast<float*>(k.omega_hi);
      float* const wlo = static_cast<float*>(k.omega_lo);
      T* const chi = F<T>(k.chi);
      // a tile farther than radius + 2 w from the body centre (z_cm, 0) has
      // mask 0 at every cell (phi < -w) and adds nothing to the drag: the
      // per-cell mask is skipped there (the same values)
      bool near = sediment;
      T zc = T(0), rbody = T(0), blendw = T(0), zcol = T(0);
      if constexpr (sizeof(T) == 8) {
        zc = scalar<T>(k, SF_ZCM);
        rbody = scalar<T>(k, SF_RBODY);
        blendw = scalar<T>(k, SF_BLENDW);
        zcol = (sediment && gjm < nz) ? CF<T>(k.zw)[gjm] : T(0);
        if (sediment) {
          const T* zw = CF<T>(k.zw);
          const T zlo = zw[j0], zhi = zw[min(j0 + TX, nz) - 1];
          const T rlo = rowf[2][1];  // r of row i0
          const T dz = zc < zlo ? zlo - zc : (zc > zhi ? zc - zhi : T(0));
          const T reach = rbody + T(2) * blendw;
          near = dz * dz + rlo * rlo <= reach * reach;
        }
      } else if (sediment) {
        // in cells: centre column S, radius R, blend W
        const float sc = scalar<T>(k, SF_S_HI);
        const float zlo = (float)j0 + 0.5f, zhi = (float)(min(j0 + TX, nz) - 1) + 0.5f;
        const float dz = sc < zlo ? zlo - sc : (sc > zhi ? sc - zhi : 0.0f);
        const float rlo = (float)i0 + 0.5f;
        const float reach = scalar<T>(k, SF_R_HI) + 2.0f * scalar<T>(k, SF_W) + 1.0f;
        near = dz * dz + rlo * rlo <= reach * reach;
      }
      const bool jin = gjm < nz, jint = gjm >= 1 && gjm < nz - 1;
      const int p0 = AD_RC * grp;
      int d = ad_tp(p0, qm);
      T s_ = tp[d - AD_SW], c_ = tp[d];
#pragma unroll
      for (int m = 0; m < AD_RC; ++m, d += AD_SW) {
        const int pr = p0 + m, gi = i0 + pr;
        const T n_ = tp[d + AD_SW];
        if (jin && gi < nr) {
          const int c = gi * nz + gjm;
          T v = wa[ad_wa(pr, qm)];
          if (jint && gi >= 1 && gi < nr - 1) {
            const T ee = tp[d + 1], ww = tp[d - 1];
            const T lap = rk2_lap<T>(n_, s_, ee, ww, c_, inv_dx2, rowf[0][pr + 1],
                                     rowf[1][pr + 1]);
            v = v + c2 * lap;
          }
          wout[c] = v;
          if constexpr (sizeof(T) == 4) {
            if (whi) {
              float hi, lo;
              axi_tc::tf32_split((float)v, hi, lo);
              whi[c] = hi;
              wlo[c] = lo;
            }
          }
          if (sediment) {
            // mask at the body position of this step (falling_rigid_sphere.py:156-157),
            // then the drag integrand with the new mask (:164-173)
            if (near) {
              const T rr = rowf[2][pr + 1];
              T ch;
              if constexpr (sizeof(T) == 8) {
                ch = sphere_mask<T>(zcol, rr, zc, rbody, blendw);
                cd_part += rr * ch * sz[ad_box(pr, qm)];
              } else {
                ch = sphere_mask_cells(gi, gjm, scalar<T>(k, SF_S_HI), scalar<T>(k, SF_S_LO),
                                       scalar<T>(k, SF_R_HI), scalar<T>(k, SF_R_LO),
                                       scalar<T>(k, SF_W));
                cd_part += rr * ch * sz[ad_box(pr, qm)];
              }
              chi[c] = ch;
            } else {
              chi[c] = T(0);
            }
          }
        }
        s_ = c_;
        c_ = n_;
      }
    }
    if (sediment) {
      double x = cd_part;
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if ((threadIdx.x & 31) == 0) red[it & 1][threadIdx.x >> 5] = (double)x;
    }
    // end of tile: the boxes and wa / tp may be reused from here on
    __syncthreads();
    if (threadIdx.x != 0) continue;
    if (!sediment) {
      if (tr.w == 0) {
        k.state[AXI_ST_T] += k.state[AXI_ST_DT];
        k.state[AXI_ST_STEPS] += 1.0;
      }
      continue;
    }
    const unsigned int ntiles = dev_tiles_of(k);
    double sum = 0.0;
    for (int q = 0; q < NT / 32; ++q) sum += red[it & 1][q];
    k.partials[ntiles + tr.w] = sum;
    __threadfence();
    if (atomicAdd(counter(k, 1), 1u) != 2 * ntiles - 1) continue;
    __threadfence();
    double tot = 0.0;
    for (unsigned int q = 0; q < ntiles; ++q) tot += ((volatile double*)k.partials)[ntiles + q];
    const double cd = k.cd_scale * tot;
    const double dt = k.state[AXI_ST_DT];
    // body ODE, falling_rigid_sphere.py:176-181 (FP64)
    const double ft = k.state[AXI_ST_FTOTAL];
    const double u_old = k.state[AXI_ST_UBODY];
    const double acc = -k.grav / k.rho_s + ft / k.part_mass;
    k.state[AXI_ST_UBODY] = u_old + dt * (-k.grav + ft / k.part_mass);
    k.state[AXI_ST_DIFF] = dt * acc;
    k.state[AXI_ST_ZCM] = k.state[AXI_ST_ZCM] + u_old * dt + 0.5 * dt * dt * acc;
    if (!(cd == cd) || !(ft == ft))
      atomicOr(reinterpret_cast<unsigned int*>(&k.state[AXI_ST_STATUS]), 1u << AXI_ERR_NONFINITE);
    const long long step = (long long)k.state[AXI_ST_STEPS];
    if (k.history && step < k.history_len) {
      k.history[2 * step] = dt;
      k.history[2 * step + 1] = cd;
    }
    k.state[AXI_ST_CD] = cd;
    k.state[AXI_ST_T] += dt;
    k.state[AXI_ST_STEPS] += 1.0;
  }
  if (!ok && threadIdx.x == 0) ring.drain(it, issued, err);
}

// Recomputes the TF32 hi / lo operand copy of omega from omega (after the
// caller replaced omega).
__global__ void __launch_bounds__(NT) refresh_split_kernel(const axi_case* __restrict__ cases,
                                                           const int4* __restrict__ tiles) {
  const int4 tr = tiles[blockIdx.x];
  const axi_case& k = cases[tr.x];
  if (!k.omega_hi) return;
#pragma unroll
  for (int q = 0; q < CPT; ++q) {
    const int e = threadIdx.x + q * NT;
    const int gi = tr.y + e / TX, gj = tr.z + e % TX;
    if (gi < k.nr && gj < k.nz) {
      const int c = gi * k.nz + gj;
      store_omega<float>(k, c, static_cast<const float*>(k.omega)[c]);
    }
  }
}

// ---------------------------------------------------------------------------
// Grouped SIMT GEMM over all cases: the four products of the spectral solve
// (kernels/FastDiagonalisationStokesSolver.py:137-156, association A (B C)):
//   stage 0  w1  = omega * EzinvT              (K = nz)
//   stage 1  w2  = (Er_inv_w * w1) .* inv_eig  (K = nr)
//   stage 2  w1  = w2 * EzT                    (K = nz)
//   stage 3  psi = Er * w1                     (K = nr)
// Every stage writes an (nr, nz) result, so one tile table serves all four.
// The FP64 configuration uses small register tiles so that even a single
// 256 x 512 case puts several warps on every SM sub-partition (the FP64 pipe,
// not latency, is the limit).
// ---------------------------------------------------------------------------
template <typename T> struct GemmCfg;
template <> struct GemmCfg<double> {
  static constexpr int BM = 32, BN = 32, BK = 32, RM = 2, RN = 2;
};
template <> struct GemmCfg<float> {
  static constexpr int BM = 64, BN = 64, BK = 16, RM = 4, RN = 4;
};

template <typename T>
constexpr int gemm_threads() {
  return (GemmCfg<T>::BM / GemmCfg<T>::RM) * (GemmCfg<T>::BN / GemmCfg<T>::RN);
}

template <typename T, int STAGE>
__global__ void __launch_bounds__(gemm_threads<T>())
    grouped_gemm_kernel(const axi_case* __restrict__ cases, const int4* __restrict__ tiles) {
  using C = GemmCfg<T>;
  constexpr int BM = C::BM, BN = C::BN, BK = C::BK, RM = C::RM, RN = C::RN;
  constexpr int TXG = BN / RN, NTH = gemm_threads<T>();
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN];
  const int4 tr = tiles[blockIdx.x];
  const axi_case& k = cases[tr.x];
  const int M = k.nr, N = k.nz;
  const T* A;
  const T* B;
  const T* S = nullptr;
  T* Cm;
  int K, lda;
  T* w1 = F<T>(k.gemm_work);
  T* w2 = w1 + (size_t)M * N;
  if (STAGE == 0) {
    A = CF<T>(k.omega); lda = N; B = CF<T>(k.EzinvT); K = N; Cm = w1;
  } else if (STAGE == 1) {
    A = CF<T>(k.Er_inv_w); lda = M; B = w1; K = M; Cm = w2; S = CF<T>(k.inv_eig);
  } else if (STAGE == 2) {
    A = w2; lda = N; B = CF<T>(k.EzT); K = N; Cm = w1;
  } else {
    A = CF<T>(k.Er); lda = M; B = w1; K = M; Cm = F<T>(k.psi);
  }
  const int ldb = N;
  const int tx = threadIdx.x % TXG, ty = threadIdx.x / TXG;
  const int m0 = tr.y, n0 = tr.z;
  T acc[RM][RN];
#pragma unroll
  for (int p = 0; p < RM; ++p)
#pragma unroll
    for (int q = 0; q < RN; ++q) acc[p][q] = T(0);
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int e = threadIdx.x; e < BM * BK; e += NTH) {
      const int r = e / BK, kk = e % BK;
      const int gm = m0 + r, gk = k0 + kk;
      As[kk][r] = (gm < M && gk < K) ? A[(long long)gm * lda + gk] : T(0);
    }
    for (int e = threadIdx.x; e < BK * BN; e += NTH) {
      const int kk = e / BN, cc = e % BN;
      const int gk = k0 + kk, gn = n0 + cc;
      Bs[kk][cc] = (gk < K && gn < N) ? B[(long long)gk * ldb + gn] : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < BK; ++kk) {
      T av[RM], bv[RN];
#pragma unroll
      for (int p = 0; p < RM; ++p) av[p] = As[kk][ty * RM + p];
#pragma unroll
      for (int q = 0; q < RN; ++q) bv[q] = Bs[kk][tx + q * TXG];
#pragma unroll
      for (int p = 0; p < RM; ++p)
#pragma unroll
        for (int q = 0; q < RN; ++q) acc[p][q] = fma(av[p], bv[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < RM; ++p) {
    const int gm = m0 + ty * RM + p;
    if (gm >= M) continue;
#pragma unroll
    for (int q = 0; q < RN; ++q) {
      const int gn = n0 + tx + q * TXG;
      if (gn >= N) continue;
      const long long c = (long long)gm * N + gn;
      T v = acc[p][q];
      if (S) v *= S[c];
      Cm[c] = v;
    }
  }
}

// Plan layout in device memory:
//   [axi_case x n][stencil tiles][gemm tiles]            (all plans)
//   [TcJob x 4n][tc tiles stage 0..3][error word]        (tensor-core plans)
struct PlanView {
  const axi_case* cases;
  const int4* stencil;
  const int4* gemm;
  const CUtensorMap* maps;
  const axi_tc::TcJob* jobs;
  const int4* tc_tiles[4];
  const axi_dct::DctJob* dct_jobs;  // forward jobs, then inverse jobs (n_cases each)
  const int4* dct_items;
  const axi_dct64::Job* dct64_jobs;  // double engine: forward, then inverse jobs
  int* err;
};

inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
inline size_t align128(size_t x) { return (x + 127) & ~size_t(127); }

struct PlanOffsets {
  size_t stencil, gemm, maps, jobs, tc_tiles[4], dct_jobs, dct_items, err, total;
};

// Plan buffer: cases | stencil tiles | SIMT GEMM tiles | stencil tensor maps
// (MAP_COUNT per case) | [tensor-core jobs | tensor-core tiles x 4] | error word
inline PlanOffsets plan_offsets(const axi_plan_info* info) {
  PlanOffsets o;
  o.stencil = align16(info->n_cases * sizeof(axi_case));
  o.gemm = o.stencil + (size_t)info->n_stencil_tiles * sizeof(int4);
  size_t end = o.gemm + (size_t)info->n_gemm_tiles * sizeof(int4);
  o.maps = align128(end);
  end = o.maps + (size_t)MAP_COUNT * info->n_cases * sizeof(CUtensorMap);
  if (info->flags & AXI_PLAN_TENSOR_CORES) {
    o.jobs = align128(end);
    end = o.jobs + (size_t)4 * info->n_cases * sizeof(axi_tc::TcJob);
    for (int st = 0; st < 4; ++st) {
      o.tc_tiles[st] = align16(end);
      end = o.tc_tiles[st] + (size_t)info->n_tc_tiles[st] * sizeof(int4);
    }
  } else {
    o.jobs = 0;
    for (int st = 0; st < 4; ++st) o.tc_tiles[st] = 0;
  }
  if (info->flags & AXI_PLAN_DCT_Z) {
    o.dct_jobs = align128(end);
    const size_t job_bytes =
        info->elem_bytes == 8 ? sizeof(axi_dct64::Job) : sizeof(axi_dct::DctJob);
    end = o.dct_jobs + (size_t)2 * info->n_cases * job_bytes;
    o.dct_items = align16(end);
    end = o.dct_items + (size_t)info->n_dct_items * sizeof(int4);
  } else {
    o.dct_jobs = o.dct_items = 0;
  }
  o.err = align16(end);
  end = o.err + 16;
  o.total = align16(end);
  return o;
}

inline PlanView plan_view(const void* plan_dev, const axi_plan_info* info) {
  const char* base = static_cast<const char*>(plan_dev);
  const PlanOffsets o = plan_offsets(info);
  PlanView v;
  v.cases = reinterpret_cast<const axi_case*>(base);
  v.stencil = reinterpret_cast<const int4*>(base + o.stencil);
  v.gemm = reinterpret_cast<const int4*>(base + o.gemm);
  v.maps = reinterpret_cast<const CUtensorMap*>(base + o.maps);
  const bool tc = (info->flags & AXI_PLAN_TENSOR_CORES) != 0;
  v.jobs = tc ? reinterpret_cast<const axi_tc::TcJob*>(base + o.jobs) : nullptr;
  for (int st = 0; st < 4; ++st)
    v.tc_tiles[st] = tc ? reinterpret_cast<const int4*>(base + o.tc_tiles[st]) : nullptr;
  const bool dct = (info->flags & AXI_PLAN_DCT_Z) != 0;
  const bool dbl = info->elem_bytes == 8;
  v.dct_jobs =
      (dct && !dbl) ? reinterpret_cast<const axi_dct::DctJob*>(base + o.dct_jobs) : nullptr;
  v.dct64_jobs =
      (dct && dbl) ? reinterpret_cast<const axi_dct64::Job*>(base + o.dct_jobs) : nullptr;
  v.dct_items = dct ? reinterpret_cast<const int4*>(base + o.dct_items) : nullptr;
  v.err = reinterpret_cast<int*>(const_cast<char*>(base) + o.err);
  return v;
}

// Tensor-core form of the four spectral products of one case (operands
// K-major): X = Ez^-1 * omega^T ... written as C = A * B^T per stage:
//   stage 0  X (nz, nr) = Ezinv (nz, nz) * [omega (nr, nz)]^T      -> split
//   stage 1  Y (nr, nz) = (ErIw (nr, nr) * [X]^T) .* inv_eig        -> split
//   stage 2  X (nz, nr) = Ez (nz, nz) * [Y]^T                       -> split
//   stage 3  psi (nr, nz) = Er (nr, nr) * [X]^T                     -> plain
// i.e. psi = E_r ((E_r^-1 diag(r) omega E_z^-T) .* inv_eig) E_z^T as in
// kernels/FastDiagonalisationStokesSolver.py:137-156.
// With `dct`, stages 0 and 2 run as z transforms (build_dct_jobs) and stage 1
// writes its scaled result plain for the inverse transform.
int build_tc_jobs(const axi_case& k, axi_tc::TcJob job[4], bool dct, bool refine) {
  const int nr = k.nr, nz = k.nz;
  const float* const* b = reinterpret_cast<const float* const*>(k.tc_basis);
  float* const* w = reinterpret_cast<float* const*>(k.tc_work);
  memset(job, 0, 4 * sizeof(axi_tc::TcJob));
  if (dct) {
    AXI_TRY(axi_tc::encode_operand(&job[1].a_hi, b[2], nr, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&job[1].a_lo, b[3], nr, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&job[1].b_hi, w[0], nz, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&job[1].b_lo, w[1], nz, nr, nr));
    // the inverse spectrum is applied by the inverse transform as it reads
    // the rows (the same float product), keeping this epilogue a plain store
    job[1].c = w[2];
    job[1].M = nr; job[1].N = nz; job[1].K = nr; job[1].ldc = nz;
    job[1].mode = axi_tc::MODE_PLAIN;
    AXI_TRY(axi_tc::encode_operand(&job[3].a_hi, b[6], nr, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&job[3].a_lo, b[7], nr, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&job[3].b_hi, w[0], nz, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&job[3].b_lo, w[1], nz, nr, nr));
    job[3].c = static_cast<float*>(k.psi); job[3].M = nr; job[3].N = nz;
    job[3].K = nr; job[3].ldc = nz; job[3].mode = axi_tc::MODE_PLAIN;
    if (refine) {
      // the solve of the residual is the correction, added to the pair
      // (psi, psi_lo) with its rounding kept in psi_lo
      job[3].c_lo = static_cast<float*>(k.psi_lo);
      job[3].mode = axi_tc::MODE_PAIR_ADD;
    }
    // products store their tiles by TMA where they overwrite (outputs 16-byte
    // aligned, nz % 4 == 0)
    if (!axi_tc::encode_output(&job[1]) || (!refine && !axi_tc::encode_output(&job[3]))) {
      axi::set_error("plan: tensor-core output map rejected (nz %d)", nz);
      return AXI_ERR_INVALID;
    }
    return AXI_OK;
  }
  // stage 0
  AXI_TRY(axi_tc::encode_operand(&job[0].a_hi, b[0], nz, nz, nz));
  AXI_TRY(axi_tc::encode_operand(&job[0].a_lo, b[1], nz, nz, nz));
  AXI_TRY(axi_tc::encode_operand(&job[0].b_hi, static_cast<const float*>(k.omega_hi), nr, nz, nz));
  AXI_TRY(axi_tc::encode_operand(&job[0].b_lo, static_cast<const float*>(k.omega_lo), nr, nz, nz));
  job[0].c = w[0]; job[0].c_lo = w[1]; job[0].M = nz; job[0].N = nr; job[0].K = nz;
  job[0].ldc = nr; job[0].mode = axi_tc::MODE_SPLIT;
  // stage 1
  AXI_TRY(axi_tc::encode_operand(&job[1].a_hi, b[2], nr, nr, nr));
  AXI_TRY(axi_tc::encode_operand(&job[1].a_lo, b[3], nr, nr, nr));
  AXI_TRY(axi_tc::encode_operand(&job[1].b_hi, w[0], nz, nr, nr));
  AXI_TRY(axi_tc::encode_operand(&job[1].b_lo, w[1], nz, nr, nr));
  job[1].c = w[2]; job[1].c_lo = w[3]; job[1].scale = static_cast<const float*>(k.inv_eig);
  job[1].M = nr; job[1].N = nz; job[1].K = nr; job[1].ldc = nz;
  job[1].mode = axi_tc::MODE_SCALE_SPLIT;
  // stage 2
  AXI_TRY(axi_tc::encode_operand(&job[2].a_hi, b[4], nz, nz, nz));
  AXI_TRY(axi_tc::encode_operand(&job[2].a_lo, b[5], nz, nz, nz));
  AXI_TRY(axi_tc::encode_operand(&job[2].b_hi, w[2], nr, nz, nz));
  AXI_TRY(axi_tc::encode_operand(&job[2].b_lo, w[3], nr, nz, nz));
  job[2].c = w[0]; job[2].c_lo = w[1]; job[2].M = nz; job[2].N = nr; job[2].K = nz;
  job[2].ldc = nr; job[2].mode = axi_tc::MODE_SPLIT;
  // stage 3
  AXI_TRY(axi_tc::encode_operand(&job[3].a_hi, b[6], nr, nr, nr));
  AXI_TRY(axi_tc::encode_operand(&job[3].a_lo, b[7], nr, nr, nr));
  AXI_TRY(axi_tc::encode_operand(&job[3].b_hi, w[0], nz, nr, nr));
  AXI_TRY(axi_tc::encode_operand(&job[3].b_lo, w[1], nz, nr, nr));
  job[3].c = static_cast<float*>(k.psi); job[3].c_lo = nullptr; job[3].M = nr; job[3].N = nz;
  job[3].K = nr; job[3].ldc = nz; job[3].mode = axi_tc::MODE_PLAIN;
  if (!axi_tc::encode_output(&job[3])) {
    axi::set_error("plan: tensor-core output map rejected (nz %d)", nz);
    return AXI_ERR_INVALID;
  }
  return AXI_OK;
}

// z transforms of one case: forward (DCT-II of the rows of omega into the
// X operand pair) and inverse (DCT-III of the rows of the plain stage-1
// result Y into the X operand pair of stage 3).
int build_dct_jobs(const axi_case& k, axi_dct::DctJob* fwd, axi_dct::DctJob* inv, bool refine) {
  axi_dct::DctJob j;
  memset(&j, 0, sizeof(j));
  j.N = k.nz;
  j.rows = k.nr;
  if (!axi_dct::plan_radices(k.nz, j.radix, &j.nstages)) {
    axi::set_error("plan: nz %d has no DCT plan (even, factors 2 and 3 only, <= %d)", k.nz,
                   axi_dct::ELEMS);
    return AXI_ERR_INVALID;
  }
  const char* t = static_cast<const char*>(k.dct_table);
  j.twiddle = reinterpret_cast<const float2*>(t);
  j.rot = reinterpret_cast<const float2*>(t + (size_t)8 * k.nz);
  float* const* w = reinterpret_cast<float* const*>(k.tc_work);
  j.out_hi = w[0];
  j.out_lo = w[1];
  *fwd = j;
  fwd->in = static_cast<const float*>(k.omega);
  fwd->scale = reinterpret_cast<const float*>(t + (size_t)16 * k.nz);
  if (refine) {
    // the residual omega - (A psi) / r of the psi the case holds
    fwd->psi = static_cast<const float*>(k.psi);
    fwd->psi_lo = static_cast<const float*>(k.psi_lo);
    fwd->rinv2dx = static_cast<const float*>(k.rinv2dx);
    fwd->rinv2 = static_cast<const float*>(k.rinv2);
    fwd->two_over_dx = (float)(2.0 / k.dx);
    fwd->inv_2dx = (float)(0.5 / k.dx);
  }
  *inv = j;
  inv->in = w[2];
  inv->scale = reinterpret_cast<const float*>(t + (size_t)20 * k.nz);
  inv->row_scale = static_cast<const float*>(k.inv_eig);
  return AXI_OK;
}

inline int dct_items_of(const axi_case& k) {
  const int r = axi_dct::rows_for(k.nz);
  return (k.nr + r - 1) / r;
}

// Double engine: z transforms of one case on the SIMT product buffers
// (gemm_work = w1 | w2, each (nr, nz)): forward omega -> w1 (in place of the
// E_z^-T product), inverse w2 -> w1 (in place of the E_z^T product). The
// table k.dct_table holds doubles: exp(-2 pi i m / nz) as (cos, sin),
// (cos, sin)(pi k / 2 nz), c_k, 1 / c_k.
int build_dct64_jobs(const axi_case& k, axi_dct64::Job* fwd, axi_dct64::Job* inv) {
  axi_dct64::Job j;
  memset(&j, 0, sizeof(j));
  j.N = k.nz;
  j.rows = k.nr;
  if (!axi_dct64::plan_radices(k.nz, j.radix, &j.nstages)) {
    axi::set_error("plan: nz %d has no double DCT plan (even, factors 2 and 3 only, <= %d)",
                   k.nz, axi_dct64::ELEMS);
    return AXI_ERR_INVALID;
  }
  const double* t = static_cast<const double*>(k.dct_table);
  j.twiddle = reinterpret_cast<const double2*>(t);
  j.rot = reinterpret_cast<const double2*>(t + (size_t)2 * k.nz);
  double* w1 = static_cast<double*>(k.gemm_work);
  double* w2 = w1 + (size_t)k.nr * k.nz;
  *fwd = j;
  fwd->in = static_cast<const double*>(k.omega);
  fwd->out = w1;
  fwd->scale = t + (size_t)4 * k.nz;
  *inv = j;
  inv->in = w2;
  inv->out = w1;
  inv->scale = t + (size_t)5 * k.nz;
  return AXI_OK;
}

inline int dct64_items_of(const axi_case& k) {
  const int r = axi_dct64::rows_per_item(k.nz);
  return (k.nr + r - 1) / r;
}

inline int tc_tiles_of(const axi_case& k, int stage) {
  const int M = (stage % 2 == 0) ? k.nz : k.nr;
  const int N = (stage % 2 == 0) ? k.nr : k.nz;
  return ((M + axi_tc::BM - 1) / axi_tc::BM) * ((N + axi_tc::BN - 1) / axi_tc::BN);
}

enum { PH_KILL = 0, PH_TRANSFORM = 1, PH_VEL_MAX = 2, PH_PENALISE = 3, PH_ADVECT_DIFFUSE = 4,
       PH_COUNT = 5,
       // the four launches of PH_TRANSFORM one at a time (timing): z product
       // or transform, radial product, z product or inverse transform, radial
       PH_TRANSFORM_PART0 = 5, PH_PARTS_END = 9 };

// The persistent stencil kernels reserve their dynamic shared memory once per
// process and run as many blocks as fit on every SM (at most one block per
// tile).
template <typename T>
int stencil_attrs() {
  static int status = -1;
  if (status < 0) {
    bool pair_ok = true;
    if constexpr (sizeof(T) == 4)
      pair_ok = cudaFuncSetAttribute(penalise_kernel<T, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     penalise_smem<T, true>()) == cudaSuccess;
    status = (pair_ok &&
              cudaFuncSetAttribute(vel_max_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   vel_max_smem<T>()) == cudaSuccess &&
              cudaFuncSetAttribute(penalise_kernel<T, false>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   penalise_smem<T, false>()) == cudaSuccess &&
              cudaFuncSetAttribute(advect_diffuse_kernel<T>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   advect_diffuse_smem<T>()) == cudaSuccess)
                 ? AXI_OK
                 : AXI_ERR_CUDA;
    if (status != AXI_OK) axi::set_error("rigid_step: cannot reserve shared memory");
  }
  return status;
}

template <typename T>
struct StencilGrid {
  // blocks per SM of each stencil phase, measured once (slot PH_COUNT: the
  // penalise variant that reads psi as a pair)
  static int per_sm(int phase, bool pair = false) {
    static int n[PH_COUNT + 1] = {0};
    const int slot = (phase == PH_PENALISE && pair) ? PH_COUNT : phase;
    if (n[slot] == 0) {
      int b = 0;
      cudaError_t e = cudaErrorInvalidValue;
      if (phase == PH_VEL_MAX)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, vel_max_kernel<T>, NT,
                                                          vel_max_smem<T>());
      else if (phase == PH_PENALISE && pair && sizeof(T) == 4)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, penalise_kernel<T, sizeof(T) == 4>,
                                                          NT, penalise_smem<T, sizeof(T) == 4>());
      else if (phase == PH_PENALISE)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, penalise_kernel<T, false>, NT,
                                                          penalise_smem<T, false>());
      else if (phase == PH_ADVECT_DIFFUSE)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, advect_diffuse_kernel<T>, NT,
                                                          advect_diffuse_smem<T>());
      n[slot] = (e == cudaSuccess && b > 0) ? b : 1;
    }
    return n[slot];
  }
  // cap on resident blocks per SM chosen by the plan's tuning (0: none)
  static int cap(const axi_plan_info* info, int phase) {
    const int q = phase == PH_VEL_MAX ? 0 : phase == PH_PENALISE ? 1 : 2;
    return info->tune.stencil_blocks_per_sm[q];
  }
  // blocks of the phase resident on the GPU at once
  static int resident(const axi_plan_info* info, int phase, bool pair = false) {
    int b = per_sm(phase, pair);
    const int c = cap(info, phase);
    if (c > 0 && c < b) b = c;
    return b * axi::sm_count();
  }
  static int get(const axi_plan_info* info, int phase, int n_tiles, bool pair = false) {
    // ring depth 1 and no cap: one block per tile; otherwise persistent blocks
    if (cap(info, phase) <= 0 &&
        ((phase == PH_PENALISE && PN_NBUF == 1) || (phase == PH_ADVECT_DIFFUSE && AD_NBUF == 1)))
      return n_tiles;
    const int g = resident(info, phase, pair);
    return n_tiles < g ? n_tiles : g;
  }
  // L2 prefetch distance in tiles (the plan's waves of resident blocks)
  static int ahead(const axi_plan_info* info, int phase, int n_tiles, bool pair = false) {
    const int w = info->tune.prefetch_waves;
    if (w < 0) return n_tiles;
    return resident(info, phase, pair) * (w > 0 ? w : 1);
  }
};

template <typename T>
int run_phase(int phase, const axi_plan_info* info, const PlanView& v, cudaStream_t s) {
  const int nt = info->n_stencil_tiles, ng = info->n_gemm_tiles;
  switch (phase) {
    case PH_KILL:
      kill_reset_kernel<T><<<dim3(KILL_BLOCKS, info->n_cases), 256, 0, s>>>(
          v.cases, reinterpret_cast<unsigned int*>(v.err + 1));
      break;
    case PH_TRANSFORM:
      if (v.dct_jobs) {
        // z transform, radial product, inverse z transform, radial product
        AXI_TRY(axi_dct::launch(v.dct_jobs, v.dct_items, info->n_dct_items, true, s,
                                info->tune.prefetch_waves));
        AXI_TRY(axi_tc::launch(v.jobs, v.tc_tiles[1], info->n_tc_tiles[1], v.err, s,
                               info->tune.tc_ctas_percent));
        AXI_TRY(axi_dct::launch(v.dct_jobs + info->n_cases, v.dct_items, info->n_dct_items,
                                false, s, info->tune.prefetch_waves));
        AXI_TRY(axi_tc::launch(v.jobs, v.tc_tiles[3], info->n_tc_tiles[3], v.err, s,
                               info->tune.tc_ctas_percent));
        break;
      }
      if (v.jobs) {
        for (int st = 0; st < 4; ++st)
          AXI_TRY(axi_tc::launch(v.jobs, v.tc_tiles[st], info->n_tc_tiles[st], v.err, s,
                                 info->tune.tc_ctas_percent));
        break;
      }
      if (v.dct64_jobs) {
        // double: z transform, radial product, inverse z transform, radial product
        AXI_TRY(axi_dct64::launch(v.dct64_jobs, v.dct_items, info->n_dct_items, true, s));
        grouped_gemm_kernel<T, 1><<<ng, gemm_threads<T>(), 0, s>>>(v.cases, v.gemm);
        AXI_TRY(axi_dct64::launch(v.dct64_jobs + info->n_cases, v.dct_items, info->n_dct_items,
                                  false, s));
        grouped_gemm_kernel<T, 3><<<ng, gemm_threads<T>(), 0, s>>>(v.cases, v.gemm);
        break;
      }
      grouped_gemm_kernel<T, 0><<<ng, gemm_threads<T>(), 0, s>>>(v.cases, v.gemm);
      grouped_gemm_kernel<T, 1><<<ng, gemm_threads<T>(), 0, s>>>(v.cases, v.gemm);
      grouped_gemm_kernel<T, 2><<<ng, gemm_threads<T>(), 0, s>>>(v.cases, v.gemm);
      grouped_gemm_kernel<T, 3><<<ng, gemm_threads<T>(), 0, s>>>(v.cases, v.gemm);
      break;
    case PH_VEL_MAX:
      AXI_TRY(stencil_attrs<T>());
      vel_max_kernel<T><<<StencilGrid<T>::get(info, PH_VEL_MAX, nt), NT, vel_max_smem<T>(), s>>>(
          v.cases, v.stencil, nt, v.maps, v.err, info->n_cases,
          reinterpret_cast<unsigned int*>(v.err + 1));
      break;
    case PH_PENALISE:
      AXI_TRY(stencil_attrs<T>());
      if constexpr (sizeof(T) == 4) {
        if (info->flags & AXI_PLAN_REFINE) {
          // psi read as psi + psi_lo
          penalise_kernel<T, true>
              <<<StencilGrid<T>::get(info, PH_PENALISE, nt, true), NT, penalise_smem<T, true>(),
                 s>>>(v.cases, v.stencil, nt, v.maps, v.err,
                      StencilGrid<T>::ahead(info, PH_PENALISE, nt, true));
          break;
        }
      }
      penalise_kernel<T, false>
          <<<StencilGrid<T>::get(info, PH_PENALISE, nt), NT, penalise_smem<T, false>(), s>>>(
              v.cases, v.stencil, nt, v.maps, v.err,
              StencilGrid<T>::ahead(info, PH_PENALISE, nt));
      break;
    case PH_ADVECT_DIFFUSE:
      AXI_TRY(stencil_attrs<T>());
      advect_diffuse_kernel<T>
          <<<StencilGrid<T>::get(info, PH_ADVECT_DIFFUSE, nt), NT, advect_diffuse_smem<T>(), s>>>(
              v.cases, v.stencil, nt, v.maps, v.err,
              StencilGrid<T>::ahead(info, PH_ADVECT_DIFFUSE, nt));
      break;
    case PH_TRANSFORM_PART0:
    case PH_TRANSFORM_PART0 + 1:
    case PH_TRANSFORM_PART0 + 2:
    case PH_TRANSFORM_PART0 + 3: {
      const int st = phase - PH_TRANSFORM_PART0;
      if (v.dct_jobs && (st == 0 || st == 2)) {
        AXI_TRY(axi_dct::launch(st == 0 ? v.dct_jobs : v.dct_jobs + info->n_cases, v.dct_items,
                                info->n_dct_items, st == 0, s, info->tune.prefetch_waves));
      } else if (v.dct64_jobs && (st == 0 || st == 2)) {
        AXI_TRY(axi_dct64::launch(st == 0 ? v.dct64_jobs : v.dct64_jobs + info->n_cases,
                                  v.dct_items, info->n_dct_items, st == 0, s));
      } else if (v.jobs) {
        AXI_TRY(axi_tc::launch(v.jobs, v.tc_tiles[st], info->n_tc_tiles[st], v.err, s,
                                 info->tune.tc_ctas_percent));
      } else if (st == 0) {
        grouped_gemm_kernel<T, 0><<<ng, gemm_threads<T>(), 0, s>>>(v.cases, v.gemm);
      } else if (st == 1) {
        grouped_gemm_kernel<T, 1><<<ng, gemm_threads<T>(), 0, s>>>(v.cases, v.gemm);
      } else if (st == 2) {
        grouped_gemm_kernel<T, 2><<<ng, gemm_threads<T>(), 0, s>>>(v.cases, v.gemm);
      } else {
        grouped_gemm_kernel<T, 3><<<ng, gemm_threads<T>(), 0, s>>>(v.cases, v.gemm);
      }
      break;
    }
    default:
      axi::set_error("rigid_phase: unknown phase %d", phase);
      return AXI_ERR_INVALID;
  }
  return axi::launch_status("rigid_phase");
}

int validate(const axi_case* cases, int n_cases, const char* what) {
  if (n_cases <= 0 || n_cases > 65535) {
    axi::set_error("%s: invalid case count %d", what, n_cases);
    return AXI_ERR_INVALID;
  }
  for (int c = 0; c < n_cases; ++c) {
    const axi_case& k = cases[c];
    if (k.nr < 8 || k.nz < 8 || k.kill_width < 2 || k.kill_width > 8 || 2 * k.kill_width > k.nz ||
        k.kill_width > k.nr || (int64_t)k.nr * k.nz >= ((int64_t)1 << 31) || (k.nz % 4) != 0) {
      axi::set_error("%s: case %d has an unsupported grid %d x %d / kill width %d (nz must be a "
                     "multiple of 4)", what, c, k.nr, k.nz, k.kill_width);
      return AXI_ERR_INVALID;
    }
    const void* ptrs[] = {k.omega, k.psi, k.u_z, k.u_r, k.chi, k.kill_coef, k.r, k.z,
                          k.rinv2dx, k.rinv2, k.rw, k.zw, k.Er, k.Er_inv_w, k.EzinvT, k.EzT,
                          k.inv_eig, k.gemm_work, k.state, k.partials};
    for (const void* p : ptrs) {
      if (!p) {
        axi::set_error("%s: case %d has a null pointer", what, c);
        return AXI_ERR_INVALID;
      }
    }
  }
  return AXI_OK;
}

int gemm_tile_dims(int elem_bytes, int* bm, int* bn) {
  if (elem_bytes == 8) {
    *bm = GemmCfg<double>::BM;
    *bn = GemmCfg<double>::BN;
  } else if (elem_bytes == 4) {
    *bm = GemmCfg<float>::BM;
    *bn = GemmCfg<float>::BN;
  } else {
    axi::set_error("plan_init: element size must be 4 or 8 (got %d)", elem_bytes);
    return AXI_ERR_INVALID;
  }
  return AXI_OK;
}

template <typename T>
int check_info(const axi_plan_info* info, const char* what) {
  if (!info || info->elem_bytes != (int)sizeof(T) || info->n_cases <= 0) {
    axi::set_error("%s: plan was built for %d-byte fields", what, info ? info->elem_bytes : 0);
    return AXI_ERR_INVALID;
  }
  return AXI_OK;
}

template <typename T>
int rigid_step(const axi_plan_info* info, const void* plan_dev, int n_steps, cudaStream_t s,
               const char* what) {
  AXI_TRY(check_info<T>(info, what));
  const PlanView v = plan_view(plan_dev, info);
  for (int step = 0; step < n_steps; ++step)
    for (int ph = 0; ph < PH_COUNT; ++ph) AXI_TRY(run_phase<T>(ph, info, v, s));
  return axi::launch_status(what);
}

template <typename T>
int rigid_phase(const axi_plan_info* info, const void* plan_dev, int phase, cudaStream_t s) {
  AXI_TRY(check_info<T>(info, "rigid_phase"));
  return run_phase<T>(phase, info, plan_view(plan_dev, info), s);
}

}  // namespace

extern "C" int axi_plan_init(axi_case* cases, int n_cases, int elem_bytes, int flags,
                             axi_plan_info* info) {
  axi::clear_error();
  AXI_TRY(validate(cases, n_cases, "plan_init"));
  AXI_TRY(axi::check_ptr("plan_init", info, "info"));
  int bm, bn;
  AXI_TRY(gemm_tile_dims(elem_bytes, &bm, &bn));
  const bool tc = (flags & AXI_PLAN_TENSOR_CORES) != 0;
  const bool dct = (flags & AXI_PLAN_DCT_Z) != 0;
  const bool refine = (flags & AXI_PLAN_REFINE) != 0;
  if (refine && !dct) {
    axi::set_error("plan_init: refinement runs on the DCT z transform (AXI_PLAN_DCT_Z)");
    return AXI_ERR_INVALID;
  }
  for (int c = 0; refine && c < n_cases; ++c) {
    if (!cases[c].psi_lo) {
      axi::set_error("plan_init: case %d: refinement needs psi_lo", c);
      return AXI_ERR_INVALID;
    }
  }
  if (tc && elem_bytes != 4) {
    axi::set_error("plan_init: tensor-core products need float32 fields");
    return AXI_ERR_INVALID;
  }
  if (dct && !tc && elem_bytes != 8) {
    axi::set_error("plan_init: the float DCT z transform goes with the tensor-core products");
    return AXI_ERR_INVALID;
  }
  if (refine && elem_bytes != 4) {
    axi::set_error("plan_init: refinement belongs to the float engine");
    return AXI_ERR_INVALID;
  }
  const axi_tuning tune = info->tune;  // the caller's launch choices survive re-planning
  memset(info, 0, sizeof(*info));
  info->tune = tune;
  int nt = 0, ng = 0, nd = 0;
  for (int c = 0; c < n_cases; ++c) {
    const axi_case& k = cases[c];
    cases[c].stencil_tile0 = nt;
    nt += tiles_of(k);
    ng += ((k.nr + bm - 1) / bm) * ((k.nz + bn - 1) / bn);
    if (tc) {
      if ((!dct && (!k.omega_hi || !k.omega_lo)) || (k.nr % 4) || (k.nz % 4)) {
        axi::set_error("plan_init: case %d lacks tensor-core operands or nr, nz not multiples of 4",
                       c);
        return AXI_ERR_INVALID;
      }
      for (int q = 0; q < 8; ++q) {
        const bool z_basis = q == 0 || q == 1 || q == 4 || q == 5;
        if ((!k.tc_basis[q] && !(dct && z_basis)) || (q < 4 && !k.tc_work[q])) {
          axi::set_error("plan_init: case %d lacks tensor-core operand %d", c, q);
          return AXI_ERR_INVALID;
        }
      }
      int radix[axi_dct::MAX_STAGES], ns;
      if (dct && (!k.dct_table || !axi_dct::plan_radices(k.nz, radix, &ns))) {
        axi::set_error("plan_init: case %d: no DCT table or nz %d not even with factors 2, 3",
                       c, k.nz);
        return AXI_ERR_INVALID;
      }
      for (int st = 0; st < 4; ++st)
        if (!(dct && (st == 0 || st == 2))) info->n_tc_tiles[st] += tc_tiles_of(k, st);
      if (dct) nd += dct_items_of(k);
    } else if (dct) {
      // double engine: DCT z transforms around the SIMT radial products
      int radix[axi_dct64::MAX_STAGES], ns;
      if (!k.dct_table || !axi_dct64::plan_radices(k.nz, radix, &ns)) {
        axi::set_error("plan_init: case %d: no DCT table or nz %d not even with factors 2, 3 "
                       "(<= %d)", c, k.nz, axi_dct64::ELEMS);
        return AXI_ERR_INVALID;
      }
      nd += dct64_items_of(k);
    }
  }
  info->n_cases = n_cases;
  info->n_stencil_tiles = nt;
  info->n_gemm_tiles = ng;
  info->elem_bytes = elem_bytes;
  info->flags = (tc ? AXI_PLAN_TENSOR_CORES : 0) | (dct ? AXI_PLAN_DCT_Z : 0) |
                (refine ? AXI_PLAN_REFINE : 0);
  info->n_dct_items = nd;
  info->bytes = (int64_t)plan_offsets(info).total;
  return AXI_OK;
}

extern "C" int axi_plan_upload(const axi_case* cases, const axi_plan_info* info, void* plan_dev,
                               void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("plan_upload", info, "info"));
  AXI_TRY(validate(cases, info->n_cases, "plan_upload"));
  AXI_TRY(axi::check_ptr("plan_upload", plan_dev, "plan_dev"));
  int bm, bn;
  AXI_TRY(gemm_tile_dims(info->elem_bytes, &bm, &bn));
  const int n = info->n_cases;
  const size_t head = align16(n * sizeof(axi_case));
  std::string buf((size_t)info->bytes, '\0');
  memcpy(&buf[0], cases, n * sizeof(axi_case));
  int4* t = reinterpret_cast<int4*>(&buf[head]);
  int q = 0;
  for (int c = 0; c < n; ++c) {
    const axi_case& k = cases[c];
    int idx = 0;
    for (int i0 = 0; i0 < k.nr; i0 += TY)
      for (int j0 = 0; j0 < k.nz; j0 += TX) t[q++] = make_int4(c, i0, j0, idx++);
  }
  if (q != info->n_stencil_tiles) {
    axi::set_error("plan_upload: cases changed since plan_init");
    return AXI_ERR_INVALID;
  }
  for (int c = 0; c < n; ++c) {
    const axi_case& k = cases[c];
    for (int m0 = 0; m0 < k.nr; m0 += bm)
      for (int n0 = 0; n0 < k.nz; n0 += bn) t[q++] = make_int4(c, m0, n0, 0);
  }
  if (q != info->n_stencil_tiles + info->n_gemm_tiles) {
    axi::set_error("plan_upload: cases changed since plan_init");
    return AXI_ERR_INVALID;
  }
  const PlanOffsets po = plan_offsets(info);
  CUtensorMap* maps = reinterpret_cast<CUtensorMap*>(&buf[po.maps]);
  for (int c = 0; c < n; ++c) {
    const axi_case& k = cases[c];
    const int eb = info->elem_bytes;
    CUtensorMap* m = maps + MAP_COUNT * c;
    AXI_TRY(axi_tma::encode_box(m + MAP_PSI, k.psi, eb, k.nr, k.nz, PSI_ROWS, BOXW));
    AXI_TRY(axi_tma::encode_box(m + MAP_CHI, k.chi, eb, k.nr, k.nz, PSI_ROWS, BOXW));
    // penalised omega, staged by penalise in the first nr x nz elements of gemm_work
    AXI_TRY(axi_tma::encode_box(m + MAP_W, k.gemm_work, eb, k.nr, k.nz, ADV_ROWS, BOXW));
    AXI_TRY(axi_tma::encode_box(m + MAP_UZ, k.u_z, eb, k.nr, k.nz, ADV_ROWS, BOXW));
    AXI_TRY(axi_tma::encode_box(m + MAP_UR, k.u_r, eb, k.nr, k.nz, ADV_ROWS, BOXW));
    if (info->flags & AXI_PLAN_REFINE)
      AXI_TRY(axi_tma::encode_box(m + MAP_PSI_LO, k.psi_lo, eb, k.nr, k.nz, PSI_ROWS, BOXW));
  }
  if (info->flags & AXI_PLAN_TENSOR_CORES) {
    const PlanOffsets& o = po;
    axi_tc::TcJob* jobs = reinterpret_cast<axi_tc::TcJob*>(&buf[o.jobs]);
    const bool dct = (info->flags & AXI_PLAN_DCT_Z) != 0;
    const bool refine = (info->flags & AXI_PLAN_REFINE) != 0;
    for (int c = 0; c < n; ++c) AXI_TRY(build_tc_jobs(cases[c], jobs + 4 * c, dct, refine));
    if (dct) {
      axi_dct::DctJob* dj = reinterpret_cast<axi_dct::DctJob*>(&buf[o.dct_jobs]);
      int4* di = reinterpret_cast<int4*>(&buf[o.dct_items]);
      int q = 0;
      int nz_min = 1 << 30;
      for (int c = 0; c < n; ++c) {
        AXI_TRY(build_dct_jobs(cases[c], dj + c, dj + n + c, refine));
        nz_min = cases[c].nz < nz_min ? cases[c].nz : nz_min;
      }
      // item order (tuning): 0 case order with the shortest rows' items
      // last (the last wave of blocks then holds the quickest items: 10 us less
      // per pair of transforms on the 64-case ensemble), 1 plain case order,
      // 2 longest rows first
      const int order = info->tune.dct_item_order;
      std::vector<int> by_case(n);
      for (int c = 0; c < n; ++c) by_case[c] = c;
      if (order == 2)
        std::stable_sort(by_case.begin(), by_case.end(),
                         [cases](int a, int b) { return cases[a].nz > cases[b].nz; });
      for (int pass = 0; pass < 2; ++pass)
        for (int c : by_case) {
          if (order == 0 && (cases[c].nz == nz_min) != (pass == 1)) continue;
          if (order != 0 && pass == 1) continue;
          const int rows = axi_dct::rows_for(cases[c].nz);
          for (int r0 = 0; r0 < cases[c].nr; r0 += rows) di[q++] = make_int4(c, r0, 0, 0);
        }
      if (q != info->n_dct_items) {
        axi::set_error("plan_upload: cases changed since plan_init");
        return AXI_ERR_INVALID;
      }
    }
    for (int st = 0; st < 4; ++st) {
      int4* tt = reinterpret_cast<int4*>(&buf[o.tc_tiles[st]]);
      int qq = 0;
      if (dct && (st == 0 || st == 2)) continue;
      for (int c = 0; c < n; ++c) {
        const axi_case& k = cases[c];
        const int M = (st % 2 == 0) ? k.nz : k.nr;
        const int N = (st % 2 == 0) ? k.nr : k.nz;
        for (int m0 = 0; m0 < M; m0 += axi_tc::BM)
          for (int n0 = 0; n0 < N; n0 += axi_tc::BN) tt[qq++] = make_int4(4 * c + st, m0, n0, 0);
      }
      if (qq != info->n_tc_tiles[st]) {
        axi::set_error("plan_upload: cases changed since plan_init");
        return AXI_ERR_INVALID;
      }
      // tile order (tuning): 0 longest main loop first, 1 case order (the
      // k-block counts are filled in either way)
      axi_tc::order_tiles_by_k(tt, qq, jobs, info->tune.tc_tile_order == 0);
    }
  }
  if (!(info->flags & AXI_PLAN_TENSOR_CORES) && (info->flags & AXI_PLAN_DCT_Z)) {
    // double engine: z transforms as DCTs, items in case order
    axi_dct64::Job* dj = reinterpret_cast<axi_dct64::Job*>(&buf[po.dct_jobs]);
    int4* di = reinterpret_cast<int4*>(&buf[po.dct_items]);
    int q = 0;
    for (int c = 0; c < n; ++c) {
      AXI_TRY(build_dct64_jobs(cases[c], dj + c, dj + n + c));
      const int rows = axi_dct64::rows_per_item(cases[c].nz);
      for (int r0 = 0; r0 < cases[c].nr; r0 += rows) di[q++] = make_int4(c, r0, 0, 0);
    }
    if (q != info->n_dct_items) {
      axi::set_error("plan_upload: cases changed since plan_init");
      return AXI_ERR_INVALID;
    }
  }
  cudaStream_t s = axi::as_stream(stream);
  if (cudaMemcpyAsync(plan_dev, buf.data(), buf.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return axi::launch_status("plan_upload");
  return AXI_OK;
}

extern "C" int axi_rigid_refresh_operands(const axi_plan_info* info, const void* plan_dev,
                                          void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("rigid_refresh_operands", info, "info"));
  AXI_TRY(axi::check_ptr("rigid_refresh_operands", plan_dev, "plan_dev"));
  if (!(info->flags & AXI_PLAN_TENSOR_CORES) || (info->flags & AXI_PLAN_DCT_Z)) return AXI_OK;
  const PlanView v = plan_view(plan_dev, info);
  refresh_split_kernel<<<info->n_stencil_tiles, NT, 0, axi::as_stream(stream)>>>(v.cases,
                                                                                  v.stencil);
  return axi::launch_status("rigid_refresh_operands");
}

extern "C" int axi_plan_tc_status(const axi_plan_info* info, const void* plan_dev, int* tc_error,
                                  void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("plan_tc_status", info, "info"));
  AXI_TRY(axi::check_ptr("plan_tc_status", plan_dev, "plan_dev"));
  *tc_error = 0;
  const PlanView v = plan_view(plan_dev, info);
  cudaStream_t s = axi::as_stream(stream);
  if (cudaMemcpyAsync(tc_error, v.err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return axi::launch_status("plan_tc_status");
  return AXI_OK;
}

extern "C" int axi_rigid_step_f64(const axi_plan_info* info, const void* plan_dev, int n_steps,
                                  void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("rigid_step", plan_dev, "plan_dev"));
  return rigid_step<double>(info, plan_dev, n_steps, axi::as_stream(stream), "rigid_step_f64");
}

extern "C" int axi_rigid_step_f32(const axi_plan_info* info, const void* plan_dev, int n_steps,
                                  void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("rigid_step", plan_dev, "plan_dev"));
  return rigid_step<float>(info, plan_dev, n_steps, axi::as_stream(stream), "rigid_step_f32");
}

extern "C" int axi_rigid_phase_f64(const axi_plan_info* info, const void* plan_dev, int phase,
                                   void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("rigid_phase", plan_dev, "plan_dev"));
  return rigid_phase<double>(info, plan_dev, phase, axi::as_stream(stream));
}

extern "C" int axi_rigid_phase_f32(const axi_plan_info* info, const void* plan_dev, int phase,
                                   void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("rigid_phase", plan_dev, "plan_dev"));
  return rigid_phase<float>(info, plan_dev, phase, axi::as_stream(stream));
}
