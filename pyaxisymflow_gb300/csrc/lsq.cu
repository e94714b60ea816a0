// Least-squares front-marching extrapolation of the reference map (eta).
//
// core/src/extrapolate_using_least_squares.hpp:142-446 restated for the GPU:
//   sweep: every cell with current ^ target set and a known (current == 1)
//   cell among its 8 neighbours is a front cell; it fits c0 + c1 x + c2 y to
//   the known cells of a 3x3 window shifted towards the known side (start
//   codes, core/src/lstsq/ExtrapolationConfig.hpp:131-158), solves the 3x3
//   normal equations with the reference's pivoted elimination
//   (core/src/lstsq/least_squares.hpp:10-59) and evaluates the fit at the
//   cell; afterwards all front cells become known. Sweeps repeat until no
//   front cell is left.
// Within a sweep every front cell reads only known cells (the window mask is
// the pre-sweep flag), so front cells are independent and run in parallel;
// the arithmetic keeps the reference's order (no FMA) and gives the same bits.
//
// Layout: one multi-block pass collects the candidate cells (current ^
// target) into a list; one CTA then runs all sweeps over that list, with an
// iteration cap. Neighbours outside the array count as unknown; a window that
// leaves the array sets AXI_ERR_RANGE (the reference reads out of bounds).
#include "axi_common.cuh"

namespace {

constexpr int LSQ_THREADS = 1024;

struct LsqHeader {
  int n_candidates;
  int n_front;
  int status;
  int sweeps;
  // multi-block sweeps: front counts of even / odd sweeps, the done flag
  int front_count[2];
  int done;
  int pad;
};
static_assert(sizeof(LsqHeader) == 32, "header is the first 32 bytes of the work buffer");

__global__ void lsq_collect_kernel(const int16_t* __restrict__ cf, const int16_t* __restrict__ tf,
                                   long long n, LsqHeader* hdr, int* __restrict__ list) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  if (cf[k] ^ tf[k]) {
    const int slot = atomicAdd(&hdr->n_candidates, 1);
    list[slot] = (int)k;
  }
}

__device__ __forceinline__ int start_code(int positional_sum, int total_sum) {
  // ExtrapolationConfig.hpp:131-138 (code) and :143-148 (start code, grid 3)
  float t = positional_sum > 4 ? (float)(ceil(0.5 * (double)(float)positional_sum) * 2.0)
                               : (float)positional_sum;
  const int code = (int)(2.0 * (double)t / (double)total_sum);
  return (2 * code - 6) / 2;
}

// The reference's unqualified abs(double) is C's int abs(int).
__device__ __forceinline__ double int_abs(double x) {
  int i = __double2int_rz(x);
  return (double)(i < 0 ? -i : i);
}

__device__ void gauss3x2(double A[3][5], double sol[2][3]) {
  for (int i = 0; i < 3; ++i) {
    int max_row = i;
    double max_el = int_abs(A[i][i]);
    for (int k = i + 1; k < 3; ++k) {
      if (int_abs(A[k][i]) > max_el) {
        max_el = fabs(A[k][i]);
        max_row = k;
      }
    }
    for (int k = i; k < 5; ++k) {
      double t = A[max_row][k];
      A[max_row][k] = A[i][k];
      A[i][k] = t;
    }
    for (int k = i + 1; k < 3; ++k) {
      const double c = __ddiv_rn(-A[k][i], A[i][i]);
      A[k][i] = 0.0;
      for (int j = i + 1; j < 5; ++j) A[k][j] = __dadd_rn(A[k][j], __dmul_rn(c, A[i][j]));
    }
  }
  for (int comp = 0; comp < 2; ++comp) {
    for (int i = 2; i >= 0; --i) {
      sol[comp][i] = __ddiv_rn(A[i][3 + comp], A[i][i]);
      for (int k = i - 1; k >= 0; --k)
        A[k][3 + comp] = __dsub_rn(A[k][3 + comp], __dmul_rn(A[k][i], sol[comp][i]));
    }
  }
}

// Front scan of candidate cell k (extrapolate_using_least_squares.hpp:196-253):
// a cell still to be filled (current ^ target) with a known neighbour among
// its 8 is a front cell; f receives its position and start codes.
__device__ __forceinline__ bool front_cell(const int16_t* __restrict__ cf,
                                           const int16_t* __restrict__ tf, int n0, int n1, int k,
                                           int4& f) {
  // Flags only ever go 0 -> 1, so the collected list is a superset of the
  // live candidates; re-test current ^ target against the live flag.
  if ((cf[k] ^ tf[k]) == 0) return false;
  const int j = k / n1, i = k - j * n1;
  int s = 0, sx = 0, sy = 0;
  for (int jl = -1; jl <= 1; ++jl) {
    const int jj = j + jl;
    for (int il = -1; il <= 1; ++il) {
      const int ii = i + il;
      int v = 0;
      if (jj >= 0 && jj < n0 && ii >= 0 && ii < n1) v = cf[(long long)jj * n1 + ii];
      if (jl != 0 || il != 0) s += v;
      sx += v * (il + 1);
      sy += v * (jl + 1);
    }
  }
  if (s == 0) return false;
  f = make_int4(i, j, start_code(sx, s), start_code(sy, s));
  return true;
}

// Local least-squares fit of front cell f (extrapolate_using_least_squares.hpp:274-438);
// false (nothing written) when the 3x3 window leaves the grid.
__device__ __forceinline__ bool fit_cell(const int16_t* __restrict__ cf, double* __restrict__ ex,
                                         double* __restrict__ ey, const double* __restrict__ gx,
                                         const double* __restrict__ gy, int n0, int n1,
                                         int4 f) {
  const int i = f.x, j = f.y;
  const int i0 = i + f.z, j0 = j + f.w;
  if (i0 < 0 || j0 < 0 || i0 + 3 > n1 || j0 + 3 > n0) return false;
  double m[9], xm[9], ym[9], r0[9], r1[9];
  int p = 0;
  for (int jl = j0; jl < j0 + 3; ++jl) {
    const double y = gy[jl];
    for (int il = i0; il < i0 + 3; ++il, ++p) {
      const long long g = (long long)jl * n1 + il;
      const double mk = (double)cf[g];
      m[p] = mk;
      xm[p] = __dmul_rn(mk, gx[il]);
      ym[p] = __dmul_rn(mk, y);
      r0[p] = __dmul_rn(mk, ex[g]);
      r1[p] = __dmul_rn(mk, ey[g]);
    }
  }
  const double* rows[3] = {m, xm, ym};
  double A[3][5];
  for (int a = 0; a < 3; ++a) {
    for (int b = 0; b < 3; ++b) {
      double acc = 0.0;
      for (int t = 0; t < 9; ++t) acc = __dadd_rn(acc, __dmul_rn(rows[a][t], rows[b][t]));
      A[a][b] = acc;
    }
    double acc0 = 0.0, acc1 = 0.0;
    for (int t = 0; t < 9; ++t) {
      acc0 = __dadd_rn(acc0, __dmul_rn(rows[a][t], r0[t]));
      acc1 = __dadd_rn(acc1, __dmul_rn(rows[a][t], r1[t]));
    }
    A[a][3] = acc0;
    A[a][4] = acc1;
  }
  double sol[2][3];
  gauss3x2(A, sol);
  const double loc[3] = {1.0, gx[i], gy[j]};
  double e0 = 0.0, e1 = 0.0;
  for (int t = 0; t < 3; ++t) {
    e0 = __dadd_rn(e0, __dmul_rn(sol[0][t], loc[t]));
    e1 = __dadd_rn(e1, __dmul_rn(sol[1][t], loc[t]));
  }
  const long long c = (long long)j * n1 + i;
  ex[c] = e0;
  ey[c] = e1;
  return true;
}

// All remaining sweeps in one CTA: scan, fits, flag update, until no front is
// left (or the cap). Continues from the sweep count and status that earlier
// multi-block sweeps left in the header.
__global__ void __launch_bounds__(LSQ_THREADS)
    lsq_sweep_kernel(int16_t* __restrict__ cf, const int16_t* __restrict__ tf,
                     double* __restrict__ ex, double* __restrict__ ey,
                     const double* __restrict__ gx, const double* __restrict__ gy, int n0, int n1,
                     int max_sweeps, LsqHeader* hdr, const int* __restrict__ list,
                     int4* __restrict__ front) {
  __shared__ int s_front;
  __shared__ int s_status;
  if (hdr->status != AXI_OK || hdr->done) return;
  const int ncand = hdr->n_candidates;
  if (threadIdx.x == 0) s_status = AXI_OK;
  int sweeps = hdr->sweeps;
  for (;;) {
    if (threadIdx.x == 0) s_front = 0;
    __syncthreads();
    // 1. front scan
    for (int q = threadIdx.x; q < ncand; q += LSQ_THREADS) {
      int4 f;
      if (front_cell(cf, tf, n0, n1, list[q], f)) front[atomicAdd(&s_front, 1)] = f;
    }
    __syncthreads();
    const int nfront = s_front;
    if (nfront == 0) break;
    if (++sweeps > max_sweeps) {
      if (threadIdx.x == 0) s_status = AXI_ERR_NOT_CONVERGED;
      break;
    }
    // 2. local fits
    for (int q = threadIdx.x; q < nfront; q += LSQ_THREADS)
      if (!fit_cell(cf, ex, ey, gx, gy, n0, n1, front[q])) s_status = AXI_ERR_RANGE;
    __syncthreads();
    // 3. flag update (extrapolate_using_least_squares.hpp:441-444)
    for (int q = threadIdx.x; q < nfront; q += LSQ_THREADS) {
      const int4 f = front[q];
      cf[(long long)f.y * n1 + f.x] = 1;
    }
    __syncthreads();
    if (s_status != AXI_OK) break;
  }
  if (threadIdx.x == 0) {
    hdr->status = s_status;
    hdr->sweeps = sweeps;
    hdr->done = 1;
  }
}

// The same sweep spread over the GPU, three launches per sweep (scan, fits,
// flag update; a launch boundary is the barrier between them). A fixed
// number of these sweeps is issued; once no front is left (or on a failure)
// the remaining launches return at once, and lsq_sweep_kernel finishes
// whatever sweeps are still needed. Front cells of a sweep are independent
// (each reads only the flags before the sweep), so the results are the
// single-CTA kernel's.
__global__ void lsq_scan_mb_kernel(const int16_t* __restrict__ cf,
                                   const int16_t* __restrict__ tf, int n0, int n1,
                                   LsqHeader* hdr, const int* __restrict__ list,
                                   int4* __restrict__ front, int parity) {
  if (hdr->status != AXI_OK || hdr->done) return;
  const int ncand = hdr->n_candidates;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ncand; q += gridDim.x * blockDim.x) {
    int4 f;
    if (front_cell(cf, tf, n0, n1, list[q], f))
      front[atomicAdd(&hdr->front_count[parity], 1)] = f;
  }
}

__global__ void lsq_fit_mb_kernel(const int16_t* __restrict__ cf, double* __restrict__ ex,
                                  double* __restrict__ ey, const double* __restrict__ gx,
                                  const double* __restrict__ gy, int n0, int n1, int max_sweeps,
                                  LsqHeader* hdr, const int4* __restrict__ front, int parity) {
  if (hdr->status != AXI_OK || hdr->done) return;
  const int nfront = hdr->front_count[parity];
  if (nfront == 0) return;
  if (hdr->sweeps + 1 > max_sweeps) {
    // the cap: counted as one more sweep, as the single-CTA loop does
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      hdr->status = AXI_ERR_NOT_CONVERGED;
      hdr->sweeps += 1;
    }
    return;
  }
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nfront; q += gridDim.x * blockDim.x)
    if (!fit_cell(cf, ex, ey, gx, gy, n0, n1, front[q]))
      atomicCAS(&hdr->status, AXI_OK, AXI_ERR_RANGE);
}

__global__ void lsq_flag_mb_kernel(int16_t* __restrict__ cf, int n1, LsqHeader* hdr,
                                   const int4* __restrict__ front, int parity) {
  if (hdr->done || hdr->status == AXI_ERR_NOT_CONVERGED) return;
  const int nfront = hdr->front_count[parity];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    hdr->front_count[parity ^ 1] = 0;  // the next sweep's count
    if (nfront == 0)
      hdr->done = 1;
    else
      hdr->sweeps += 1;
  }
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nfront; q += gridDim.x * blockDim.x) {
    const int4 f = front[q];
    cf[(long long)f.y * n1 + f.x] = 1;
  }
}

}  // namespace

extern "C" int64_t axi_lsq_work_bytes(int n0, int n1) {
  const long long n = (long long)n0 * n1;
  return (int64_t)(sizeof(LsqHeader) + 16 + n * (long long)sizeof(int) + 16 +
                   n * (long long)sizeof(int4));
}

namespace {

// Sweeps issued as multi-block launches before the single-CTA kernel takes
// over: front marching needs about extrap_zone / dx sweeps (6 or 7 on the
// soft-sphere grids, plus one that finds no front), so these usually finish
// the extrapolation.
constexpr int MB_SWEEPS = 8;

void issue_sweeps(int16_t* cf, const int16_t* tf, double* ex, double* ey, const double* gx,
                  const double* gy, int n0, int n1, int max_sweeps, LsqHeader* hdr,
                  const int* list, int4* front, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = 2 * (sms > 0 ? sms : 1);
  for (int k = 0; k < MB_SWEEPS; ++k) {
    const int parity = k & 1;
    lsq_scan_mb_kernel<<<blocks, 256, 0, s>>>(cf, tf, n0, n1, hdr, list, front, parity);
    lsq_fit_mb_kernel<<<blocks, 128, 0, s>>>(cf, ex, ey, gx, gy, n0, n1, max_sweeps, hdr, front,
                                              parity);
    lsq_flag_mb_kernel<<<blocks, 256, 0, s>>>(cf, n1, hdr, front, parity);
  }
  lsq_sweep_kernel<<<1, LSQ_THREADS, 0, s>>>(cf, tf, ex, ey, gx, gy, n0, n1, max_sweeps, hdr,
                                             list, front);
}

int lsq_run(int16_t* cf, const int16_t* tf, double* ex, double* ey, const double* gx,
            const double* gy, int n0, int n1, int max_sweeps, void* work, int* sweeps_out,
            cudaStream_t s) {
  const char* what = "extrapolate_lsq_first_order";
  if (n0 < 1 || n1 < 1 || max_sweeps < 0) {
    axi::set_error("%s: invalid size %d x %d", what, n0, n1);
    return AXI_ERR_INVALID;
  }
  AXI_TRY(axi::check_ptrs(what, {cf, tf, ex, ey, gx, gy, work},
                          {"current_flag", "target_flag", "eta_x", "eta_y", "grid_x", "grid_y",
                           "work"}));
  const long long n = (long long)n0 * n1;
  char* base = static_cast<char*>(work);
  LsqHeader* hdr = reinterpret_cast<LsqHeader*>(base);
  int* list = reinterpret_cast<int*>(base + 16 + 16);
  size_t off = 32 + n * sizeof(int);
  off = (off + 15) & ~size_t(15);
  int4* front = reinterpret_cast<int4*>(base + off);
  if (cudaMemsetAsync(hdr, 0, sizeof(LsqHeader), s) != cudaSuccess) return axi::launch_status(what);
  lsq_collect_kernel<<<axi::ceil_div(n, 256), 256, 0, s>>>(cf, tf, n, hdr, list);
  issue_sweeps(cf, tf, ex, ey, gx, gy, n0, n1, max_sweeps, hdr, list, front, s);
  AXI_TRY(axi::launch_status(what));
  LsqHeader h;
  if (cudaMemcpyAsync(&h, hdr, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return axi::launch_status(what);
  if (sweeps_out) *sweeps_out = h.sweeps;
  if (h.status == AXI_ERR_NOT_CONVERGED) {
    axi::set_error("%s: no convergence after %d sweeps", what, max_sweeps);
  } else if (h.status == AXI_ERR_RANGE) {
    axi::set_error("%s: a 3x3 fitting window leaves the %d x %d grid", what, n0, n1);
  }
  return h.status;
}

// Folds the sweep outcome into the soft loop's state block: the status bit
// of a failure (sticky) and the largest sweep count seen.
__global__ void lsq_fold_kernel(const LsqHeader* hdr, double* state) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (hdr->status != AXI_OK)
    atomicOr(reinterpret_cast<unsigned long long*>(state + AXI_SOFT_STATUS),
             1ull << hdr->status);
  if ((double)hdr->sweeps > state[AXI_SOFT_SWEEPS]) state[AXI_SOFT_SWEEPS] = hdr->sweeps;
}

// extrapolate_eta_using_least_squares_unb.py:19-24 and
// extrapolate_using_least_squares.py:33-35: doubled (2 nr, nz) buffers, upper
// half = field, lower half = flipped mirror; flags from the doubled level set.
__global__ void lsq_prepare_kernel(const uint8_t* __restrict__ inside, const double* __restrict__ phi,
                                   const double* __restrict__ eta1, const double* __restrict__ eta2,
                                   double* __restrict__ phid, double* __restrict__ e1d,
                                   double* __restrict__ e2d, int16_t* __restrict__ cf,
                                   int16_t* __restrict__ tf, double zone, int nr, int nz) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;  // doubled row
  if (j >= nz || b >= 2 * nr) return;
  const bool upper = b >= nr;
  const int i = upper ? b - nr : nr - 1 - b;
  const long long src = (long long)i * nz + j;
  const long long dst = (long long)b * nz + j;
  const double in = inside[src] ? 1.0 : 0.0;
  const double p = -phi[src];
  const double m1 = __dmul_rn(in, eta1[src]);
  const double m2 = __dmul_rn(in, eta2[src]);
  phid[dst] = p;
  e1d[dst] = m1;
  e2d[dst] = upper ? m2 : -m2;
  cf[dst] = p < 0.0 ? 1 : 0;
  tf[dst] = p < zone ? 1 : 0;
}

__global__ void lsq_copyback_kernel(const double* __restrict__ e1d, const double* __restrict__ e2d,
                                    double* __restrict__ eta1, double* __restrict__ eta2, int nr,
                                    int nz) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= nz || i >= nr) return;
  const long long c = (long long)i * nz + j;
  const long long d = (long long)(nr + i) * nz + j;
  eta1[c] = e1d[d];
  eta2[c] = e2d[d];
}

}  // namespace

extern "C" int axi_extrapolate_lsq_first_order_f64(int16_t* current_flag,
                                                   const int16_t* target_flag, double* eta_x,
                                                   double* eta_y, const double* grid_x,
                                                   const double* grid_y, int n0, int n1,
                                                   int max_sweeps, void* work, int* sweeps_out,
                                                   void* stream) {
  axi::clear_error();
  return lsq_run(current_flag, target_flag, eta_x, eta_y, grid_x, grid_y, n0, n1, max_sweeps,
                 work, sweeps_out, axi::as_stream(stream));
}

extern "C" int axi_extrapolate_eta_with_least_squares_f64(
    const uint8_t* inside_solid, const double* ball_phi, double* eta1, double* eta2,
    double* ball_phi_double, double* eta1_double, double* eta2_double, int16_t* current_flag,
    int16_t* target_flag, double extrap_zone, int nr, int nz, const double* grid_x,
    const double* grid_y, int max_sweeps, void* work, int* sweeps_out, void* stream) {
  axi::clear_error();
  const char* what = "extrapolate_eta_with_least_squares";
  if (nr < 1 || nz < 1 || 2 * nr > 65535) {
    axi::set_error("%s: invalid grid %d x %d", what, nr, nz);
    return AXI_ERR_INVALID;
  }
  AXI_TRY(axi::check_ptrs(what,
                          {inside_solid, ball_phi, eta1, eta2, ball_phi_double, eta1_double,
                           eta2_double, current_flag, target_flag, grid_x, grid_y, work},
                          {"inside_solid", "ball_phi", "eta1", "eta2", "ball_phi_double",
                           "eta1_double", "eta2_double", "current_flag", "target_flag", "grid_x",
                           "grid_y", "work"}));
  cudaStream_t s = axi::as_stream(stream);
  dim3 g2(axi::ceil_div(nz, 128), 2 * nr);
  lsq_prepare_kernel<<<g2, 128, 0, s>>>(inside_solid, ball_phi, eta1, eta2, ball_phi_double,
                                        eta1_double, eta2_double, current_flag, target_flag,
                                        extrap_zone, nr, nz);
  AXI_TRY(axi::launch_status(what));
  AXI_TRY(lsq_run(current_flag, target_flag, eta1_double, eta2_double, grid_x, grid_y, 2 * nr, nz,
                  max_sweeps, work, sweeps_out, s));
  dim3 g1(axi::ceil_div(nz, 128), nr);
  lsq_copyback_kernel<<<g1, 128, 0, s>>>(eta1_double, eta2_double, eta1, eta2, nr, nz);
  return axi::launch_status(what);
}

// The soft loop's extrapolation without a host round trip: the same kernels
// as axi_extrapolate_eta_with_least_squares_f64; the outcome goes to
// state[AXI_SOFT_STATUS] (bit 1 << AXI_ERR_NOT_CONVERGED or AXI_ERR_RANGE) and
// state[AXI_SOFT_SWEEPS] instead of the return value.
extern "C" int axi_soft_extrapolate_eta_f64(
    const uint8_t* inside_solid, const double* ball_phi, double* eta1, double* eta2,
    double* ball_phi_double, double* eta1_double, double* eta2_double, int16_t* current_flag,
    int16_t* target_flag, double extrap_zone, int nr, int nz, const double* grid_x,
    const double* grid_y, int max_sweeps, void* work, double* state, void* stream) {
  axi::clear_error();
  const char* what = "soft_extrapolate_eta";
  if (nr < 1 || nz < 1 || 2 * nr > 65535 || max_sweeps < 0) {
    axi::set_error("%s: invalid grid %d x %d", what, nr, nz);
    return AXI_ERR_INVALID;
  }
  AXI_TRY(axi::check_ptrs(what,
                          {inside_solid, ball_phi, eta1, eta2, ball_phi_double, eta1_double,
                           eta2_double, current_flag, target_flag, grid_x, grid_y, work, state},
                          {"inside_solid", "ball_phi", "eta1", "eta2", "ball_phi_double",
                           "eta1_double", "eta2_double", "current_flag", "target_flag", "grid_x",
                           "grid_y", "work", "state"}));
  cudaStream_t s = axi::as_stream(stream);
  dim3 g2(axi::ceil_div(nz, 128), 2 * nr);
  lsq_prepare_kernel<<<g2, 128, 0, s>>>(inside_solid, ball_phi, eta1, eta2, ball_phi_double,
                                        eta1_double, eta2_double, current_flag, target_flag,
                                        extrap_zone, nr, nz);
  const int n0 = 2 * nr, n1 = nz;
  const long long n = (long long)n0 * n1;
  char* base = static_cast<char*>(work);
  LsqHeader* hdr = reinterpret_cast<LsqHeader*>(base);
  int* list = reinterpret_cast<int*>(base + 16 + 16);
  size_t off = 32 + n * sizeof(int);
  off = (off + 15) & ~size_t(15);
  int4* front = reinterpret_cast<int4*>(base + off);
  if (cudaMemsetAsync(hdr, 0, sizeof(LsqHeader), s) != cudaSuccess) return axi::launch_status(what);
  lsq_collect_kernel<<<axi::ceil_div(n, 256), 256, 0, s>>>(current_flag, target_flag, n, hdr,
                                                           list);
  issue_sweeps(current_flag, target_flag, eta1_double, eta2_double, grid_x, grid_y, n0, n1,
               max_sweeps, hdr, list, front, s);
  lsq_fold_kernel<<<1, 32, 0, s>>>(hdr, state);
  dim3 g1(axi::ceil_div(nz, 128), nr);
  lsq_copyback_kernel<<<g1, 128, 0, s>>>(eta1_double, eta2_double, eta1, eta2, nr, nz);
  return axi::launch_status(what);
}
