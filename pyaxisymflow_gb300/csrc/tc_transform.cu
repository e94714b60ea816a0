// Standalone spectral transform on the tensor cores, and the pieces of one
// step of iterative refinement around it.
//
//   out = E_r ((E_r^-1 W in E_z^-T) .* inv_eig) E_z^T
// (kernels/FastDiagonalisationStokesSolver.py:130-156 with W = diag(r);
// FastDiagonalisationPotentialSolver.py:119-145 with W = I) as four tcgen05
// 3xTF32 products in the K-major form used by the FP32 engine:
//   X (nz, nr) = Ez^-1 * in^T           -> split
//   Y (nr, nz) = (ErW * X^T) .* inv_eig -> split
//   X (nz, nr) = Ez * Y^T               -> split
//   out (nr, nz) = Er * X^T             -> plain FP32
// A refinement step computes the residual rhs - L psi of the discrete
// operator in FP64 (axi_fd_residual_f64), transforms it, and adds the
// correction in FP64 (axi_add_f32_to_f64).
#include <cstring>
#include <string>

#include "tc_gemm.cuh"

namespace {

__global__ void split_f32_kernel(const float* __restrict__ x, float* __restrict__ hi,
                                 float* __restrict__ lo, long long n) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) axi_tc::tf32_split(x[k], hi[k], lo[k]);
}

// hi = nearest TF32 of fl32(x), lo = nearest TF32 of fl32(x - hi) (remainder
// taken in double): the split of an FP64 value keeps about 23 significant bits.
__global__ void split_f64_kernel(const double* __restrict__ x, float* __restrict__ hi,
                                 float* __restrict__ lo, long long n) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    const double v = x[k];
    const float h = axi_tc::tf32_round((float)v);
    hi[k] = h;
    lo[k] = axi_tc::tf32_round((float)(v - (double)h));
  }
}

// The transform solves L psi = W rhs (W = diag(w) on rows, folded into its
// E_r^-1 W basis), so the correction it is applied to is the unweighted
// residual res = rhs - W^-1 L psi, with L = A_r (rows) + A_z (columns) given by the
// three diagonals of each 1-D operator plus the two periodic wrap entries
// A_z[0, nz-1] and A_z[nz-1, 0] (the FD matrices of
// FastDiagonalisationStokesSolver.py:41-97 after the boundary edits).
__global__ void residual_kernel(double* __restrict__ res, const double* __restrict__ rhs,
                                const double* __restrict__ psi, const double* __restrict__ w,
                                const double* __restrict__ ar, const double* __restrict__ zr,
                                int nr, int nz, double wrap0, double wrap1) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (i >= nr || j >= nz) return;
  const long long c = (long long)i * nz + j;
  // radial diagonals: ar[3 i + 0] (i, i-1), ar[3 i + 1] (i, i), ar[3 i + 2] (i, i+1)
  double lp = ar[3 * i + 1] * psi[c];
  if (i > 0) lp += ar[3 * i] * psi[c - nz];
  if (i < nr - 1) lp += ar[3 * i + 2] * psi[c + nz];
  lp += zr[3 * j + 1] * psi[c];
  if (j > 0) lp += zr[3 * j] * psi[c - 1];
  if (j < nz - 1) lp += zr[3 * j + 2] * psi[c + 1];
  if (j == 0) lp += wrap0 * psi[c + nz - 1];
  if (j == nz - 1) lp += wrap1 * psi[c - nz + 1];
  res[c] = w ? rhs[c] - lp / w[i] : rhs[c] - lp;
}

__global__ void add_kernel(double* __restrict__ y, const float* __restrict__ x, long long n) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) y[k] += (double)x[k];
}

__global__ void widen_kernel(double* __restrict__ y, const float* __restrict__ x, long long n) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) y[k] = (double)x[k];
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct PlanLayout {
  size_t jobs, tiles[4], err, total;
};

int stage_tiles(const axi_tc_transform& t, int st) {
  const int M = (st % 2 == 0) ? t.nz : t.nr;
  const int N = (st % 2 == 0) ? t.nr : t.nz;
  return ((M + axi_tc::BM - 1) / axi_tc::BM) * ((N + axi_tc::BN - 1) / axi_tc::BN);
}

PlanLayout layout(const axi_tc_transform* t, int n) {
  PlanLayout L;
  size_t o = 0;
  L.jobs = o;
  o = align_up(o + (size_t)4 * n * sizeof(axi_tc::TcJob), 128);
  for (int st = 0; st < 4; ++st) {
    int tiles = 0;
    if (t)
      for (int q = 0; q < n; ++q) tiles += stage_tiles(t[q], st);
    L.tiles[st] = o;
    o = align_up(o + (size_t)tiles * sizeof(int4), 16);
  }
  L.err = o;
  o += 16;
  L.total = align_up(o, 256);
  return L;
}

}  // namespace

extern "C" int axi_tc_transform_plan(const axi_tc_transform* t, int n, void* plan_dev,
                                     axi_tc_plan_info* info, void* stream) {
  axi::clear_error();
  const char* what = "tc_transform_plan";
  AXI_TRY(axi::check_ptr(what, t, "transforms"));
  AXI_TRY(axi::check_ptr(what, info, "info"));
  if (n <= 0) {
    axi::set_error("%s: empty transform list", what);
    return AXI_ERR_INVALID;
  }
  const PlanLayout L = layout(t, n);
  info->n = n;
  info->bytes = (int64_t)L.total;
  for (int st = 0; st < 4; ++st) {
    info->n_tiles[st] = 0;
    for (int q = 0; q < n; ++q) info->n_tiles[st] += stage_tiles(t[q], st);
  }
  if (!plan_dev) return AXI_OK;  // size query
  std::string buf(L.total, '\0');
  axi_tc::TcJob* jobs = reinterpret_cast<axi_tc::TcJob*>(&buf[L.jobs]);
  for (int q = 0; q < n; ++q) {
    const axi_tc_transform& k = t[q];
    const int nr = k.nr, nz = k.nz;
    if (nr <= 0 || nz <= 0 || nr % 4 || nz % 4) {
      axi::set_error("%s: grid %d x %d must be positive multiples of 4", what, nr, nz);
      return AXI_ERR_INVALID;
    }
    for (int b = 0; b < 8; ++b) AXI_TRY(axi::check_ptr(what, k.basis[b], "basis"));
    for (int b = 0; b < 4; ++b) AXI_TRY(axi::check_ptr(what, k.work[b], "work"));
    AXI_TRY(axi::check_ptr(what, k.in_hi, "in_hi"));
    AXI_TRY(axi::check_ptr(what, k.in_lo, "in_lo"));
    AXI_TRY(axi::check_ptr(what, k.inv_eig, "inv_eig"));
    AXI_TRY(axi::check_ptr(what, k.out, "out"));
    axi_tc::TcJob* j = jobs + 4 * q;
    memset(j, 0, 4 * sizeof(axi_tc::TcJob));
    AXI_TRY(axi_tc::encode_operand(&j[0].a_hi, k.basis[0], nz, nz, nz));
    AXI_TRY(axi_tc::encode_operand(&j[0].a_lo, k.basis[1], nz, nz, nz));
    AXI_TRY(axi_tc::encode_operand(&j[0].b_hi, k.in_hi, nr, nz, nz));
    AXI_TRY(axi_tc::encode_operand(&j[0].b_lo, k.in_lo, nr, nz, nz));
    j[0].c = k.work[0]; j[0].c_lo = k.work[1]; j[0].M = nz; j[0].N = nr; j[0].K = nz;
    j[0].ldc = nr; j[0].mode = axi_tc::MODE_SPLIT;
    AXI_TRY(axi_tc::encode_operand(&j[1].a_hi, k.basis[2], nr, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&j[1].a_lo, k.basis[3], nr, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&j[1].b_hi, k.work[0], nz, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&j[1].b_lo, k.work[1], nz, nr, nr));
    j[1].c = k.work[2]; j[1].c_lo = k.work[3]; j[1].scale = k.inv_eig; j[1].M = nr;
    j[1].N = nz; j[1].K = nr; j[1].ldc = nz; j[1].mode = axi_tc::MODE_SCALE_SPLIT;
    AXI_TRY(axi_tc::encode_operand(&j[2].a_hi, k.basis[4], nz, nz, nz));
    AXI_TRY(axi_tc::encode_operand(&j[2].a_lo, k.basis[5], nz, nz, nz));
    AXI_TRY(axi_tc::encode_operand(&j[2].b_hi, k.work[2], nr, nz, nz));
    AXI_TRY(axi_tc::encode_operand(&j[2].b_lo, k.work[3], nr, nz, nz));
    j[2].c = k.work[0]; j[2].c_lo = k.work[1]; j[2].M = nz; j[2].N = nr; j[2].K = nz;
    j[2].ldc = nr; j[2].mode = axi_tc::MODE_SPLIT;
    AXI_TRY(axi_tc::encode_operand(&j[3].a_hi, k.basis[6], nr, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&j[3].a_lo, k.basis[7], nr, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&j[3].b_hi, k.work[0], nz, nr, nr));
    AXI_TRY(axi_tc::encode_operand(&j[3].b_lo, k.work[1], nz, nr, nr));
    j[3].c = k.out; j[3].M = nr; j[3].N = nz; j[3].K = nr; j[3].ldc = nz;
    j[3].mode = axi_tc::MODE_PLAIN;
  }
  // stage 3 stores its tiles by TMA when every case's output allows it (the
  // jobs of one launch must agree)
  bool all_tma = true;
  for (int q = 0; q < n && all_tma; ++q)
    all_tma = axi_tc::encode_output(&reinterpret_cast<axi_tc::TcJob*>(&buf[L.jobs])[4 * q + 3]);
  if (!all_tma)
    for (int q = 0; q < n; ++q) reinterpret_cast<axi_tc::TcJob*>(&buf[L.jobs])[4 * q + 3].c_tma = 0;
  for (int st = 0; st < 4; ++st) {
    int4* tt = reinterpret_cast<int4*>(&buf[L.tiles[st]]);
    int qq = 0;
    for (int q = 0; q < n; ++q) {
      const int M = (st % 2 == 0) ? t[q].nz : t[q].nr;
      const int N = (st % 2 == 0) ? t[q].nr : t[q].nz;
      for (int m0 = 0; m0 < M; m0 += axi_tc::BM)
        for (int n0 = 0; n0 < N; n0 += axi_tc::BN) tt[qq++] = make_int4(4 * q + st, m0, n0, 0);
    }
    axi_tc::order_tiles_by_k(tt, qq, jobs);
  }
  cudaStream_t s = axi::as_stream(stream);
  if (cudaMemcpyAsync(plan_dev, buf.data(), buf.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return axi::launch_status(what);
  return AXI_OK;
}

extern "C" int axi_tc_transform_run(const axi_tc_plan_info* info, const void* plan_dev,
                                    void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("tc_transform_run", info, "info"));
  AXI_TRY(axi::check_ptr("tc_transform_run", plan_dev, "plan_dev"));
  const PlanLayout L = layout(nullptr, info->n);
  // tile offsets depend on the tile counts recorded in info
  size_t o = align_up((size_t)4 * info->n * sizeof(axi_tc::TcJob), 128);
  size_t toff[4];
  for (int st = 0; st < 4; ++st) {
    toff[st] = o;
    o = align_up(o + (size_t)info->n_tiles[st] * sizeof(int4), 16);
  }
  const char* base = static_cast<const char*>(plan_dev);
  const axi_tc::TcJob* jobs = reinterpret_cast<const axi_tc::TcJob*>(base + L.jobs);
  int* err = reinterpret_cast<int*>(const_cast<char*>(base) + o);
  cudaStream_t s = axi::as_stream(stream);
  for (int st = 0; st < 4; ++st)
    AXI_TRY(axi_tc::launch(jobs, reinterpret_cast<const int4*>(base + toff[st]),
                           info->n_tiles[st], err, s));
  return AXI_OK;
}

extern "C" int axi_tc_transform_status(const axi_tc_plan_info* info, const void* plan_dev,
                                       int* tc_error, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("tc_transform_status", info, "info"));
  size_t o = align_up((size_t)4 * info->n * sizeof(axi_tc::TcJob), 128);
  for (int st = 0; st < 4; ++st) o = align_up(o + (size_t)info->n_tiles[st] * sizeof(int4), 16);
  cudaStream_t s = axi::as_stream(stream);
  if (cudaMemcpyAsync(tc_error, static_cast<const char*>(plan_dev) + o, sizeof(int),
                      cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return axi::launch_status("tc_transform_status");
  return AXI_OK;
}

extern "C" int axi_tc_split_f32(float* hi, float* lo, const float* x, int64_t n, void* stream) {
  axi::clear_error();
  if (n <= 0) return AXI_OK;
  AXI_TRY(axi::check_ptrs("tc_split_f32", {hi, lo, x}, {"hi", "lo", "x"}));
  split_f32_kernel<<<axi::ceil_div(n, 256), 256, 0, axi::as_stream(stream)>>>(x, hi, lo, n);
  return axi::launch_status("tc_split_f32");
}

extern "C" int axi_tc_split_f64(float* hi, float* lo, const double* x, int64_t n, void* stream) {
  axi::clear_error();
  if (n <= 0) return AXI_OK;
  AXI_TRY(axi::check_ptrs("tc_split_f64", {hi, lo, x}, {"hi", "lo", "x"}));
  split_f64_kernel<<<axi::ceil_div(n, 256), 256, 0, axi::as_stream(stream)>>>(x, hi, lo, n);
  return axi::launch_status("tc_split_f64");
}

extern "C" int axi_fd_residual_f64(double* res, const double* rhs, const double* psi,
                                   const double* row_weight, const double* ar, const double* az,
                                   int nr, int nz, double wrap0, double wrap1, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_grid("fd_residual", nr, nz, 1, 2));
  if (nr > 65535) {
    axi::set_error("fd_residual: nr %d too large", nr);
    return AXI_ERR_INVALID;
  }
  // row_weight may be null (no weight)
  AXI_TRY(axi::check_ptrs("fd_residual", {res, rhs, psi, ar, az},
                          {"residual", "rhs", "psi", "op_r", "op_z"}));
  dim3 grid(axi::ceil_div(nz, 256), nr);
  residual_kernel<<<grid, 256, 0, axi::as_stream(stream)>>>(res, rhs, psi, row_weight, ar, az, nr,
                                                            nz, wrap0, wrap1);
  return axi::launch_status("fd_residual");
}

extern "C" int axi_add_f32_to_f64(double* y, const float* x, int64_t n, void* stream) {
  axi::clear_error();
  if (n <= 0) return AXI_OK;
  AXI_TRY(axi::check_ptrs("add_f32_to_f64", {y, x}, {"y", "x"}));
  add_kernel<<<axi::ceil_div(n, 256), 256, 0, axi::as_stream(stream)>>>(y, x, n);
  return axi::launch_status("add_f32_to_f64");
}

extern "C" int axi_widen_f32_to_f64(double* y, const float* x, int64_t n, void* stream) {
  axi::clear_error();
  if (n <= 0) return AXI_OK;
  AXI_TRY(axi::check_ptrs("widen_f32_to_f64", {y, x}, {"y", "x"}));
  widen_kernel<<<axi::ceil_div(n, 256), 256, 0, axi::as_stream(stream)>>>(y, x, n);
  return axi::launch_status("widen_f32_to_f64");
}
