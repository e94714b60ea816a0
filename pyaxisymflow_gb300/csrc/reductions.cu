// Body-force integrals (FP64 accumulation, fixed reduction order).
//
// kernels/compute_forces.py:14-15: F_pen = rho_f lam sum(R chi (u_z - U)), F_un = diff vol / dt
// kernels/force_projection.py:12-13: U = sum(rho chi u R) / sum(rho chi R)
//
// Pass 1: a fixed grid of blocks, each summing a grid-strided slice in double
// and writing one partial per quantity. Pass 2: one block folds the partials
// in index order and applies the scalar formula. The grid size depends only on
// n, so the bits are reproducible from call to call.
#include "axi_common.cuh"

namespace {

constexpr int RED_THREADS = 256;
constexpr int RED_MAX_BLOCKS = 1024;

inline int red_blocks(long long n) {
  long long b = (n + RED_THREADS * 8 - 1) / (RED_THREADS * 8);
  if (b < 1) b = 1;
  if (b > RED_MAX_BLOCKS) b = RED_MAX_BLOCKS;
  return (int)b;
}

template <int NQ>
__device__ __forceinline__ void block_sum(double (&v)[NQ], double* out) {
  __shared__ double sh[NQ][RED_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[q][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double x = lane < RED_THREADS / 32 ? sh[q][lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) out[q] = x;
    }
  }
}

template <typename T>
__global__ void force_partials_kernel(const T* __restrict__ R, const T* __restrict__ chi,
                                      const T* __restrict__ uz, double U, long long n,
                                      double* __restrict__ partials) {
  double v[1] = {0.0};
  for (long long k = (long long)blockIdx.x * RED_THREADS + threadIdx.x; k < n;
       k += (long long)gridDim.x * RED_THREADS) {
    const double rc = (double)R[k] * (double)chi[k];
    v[0] += rc * ((double)uz[k] - U);
  }
  block_sum<1>(v, partials + blockIdx.x);
}

template <typename T>
__global__ void projection_partials_kernel(double rho, const T* __restrict__ chi,
                                           const T* __restrict__ uz, const T* __restrict__ ur,
                                           const T* __restrict__ R, long long n,
                                           double* __restrict__ partials) {
  double v[3] = {0.0, 0.0, 0.0};
  for (long long k = (long long)blockIdx.x * RED_THREADS + threadIdx.x; k < n;
       k += (long long)gridDim.x * RED_THREADS) {
    const double rc = rho * (double)chi[k];
    const double r = (double)R[k];
    v[0] += rc * (double)uz[k] * r;
    v[1] += rc * (double)ur[k] * r;
    v[2] += rc * r;
  }
  double tmp[3];
  block_sum<3>(v, tmp);
  if (threadIdx.x == 0) {
    partials[3 * blockIdx.x + 0] = tmp[0];
    partials[3 * blockIdx.x + 1] = tmp[1];
    partials[3 * blockIdx.x + 2] = tmp[2];
  }
}

// mode 0: force on body -> out = {rho_f lam S, diff vol / dt}
// mode 1: projection -> out = {S0 / S2, S1 / S2}
__global__ void finish_kernel(const double* __restrict__ partials, int nblocks, int nq, int mode,
                              double c0, double c1, double* __restrict__ out) {
  double v[3] = {0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblocks; b += RED_THREADS)
    for (int q = 0; q < nq; ++q) v[q] += partials[(long long)b * nq + q];
  double s[3];
  block_sum<3>(v, s);
  if (threadIdx.x == 0) {
    if (mode == 0) {
      out[0] = c0 * s[0];
      out[1] = c1;
    } else {
      out[0] = s[0] / s[2];
      out[1] = s[1] / s[2];
    }
  }
}

template <typename T>
int force_on_body(const T* R, const T* chi, double rho_f, double lam, const T* uz, double U,
                  double vol, double dt, double diff, long long n, double* partials, double* out,
                  cudaStream_t s) {
  if (n <= 0) {
    axi::set_error("compute_force_on_body: empty field");
    return AXI_ERR_INVALID;
  }
  AXI_TRY(axi::check_ptrs("compute_force_on_body", {R, chi, uz, partials, out},
                          {"R", "char_func", "u_z", "partials", "out"}));
  const int nb = red_blocks(n);
  force_partials_kernel<T><<<nb, RED_THREADS, 0, s>>>(R, chi, uz, U, n, partials);
  finish_kernel<<<1, RED_THREADS, 0, s>>>(partials, nb, 1, 0, rho_f * lam, (diff * vol) / dt, out);
  return axi::launch_status("compute_force_on_body");
}

template <typename T>
int projection(double rho, const T* chi, const T* uz, const T* ur, const T* R, long long n,
               double* partials, double* out, cudaStream_t s) {
  if (n <= 0) {
    axi::set_error("force_projection: empty field");
    return AXI_ERR_INVALID;
  }
  AXI_TRY(axi::check_ptrs("force_projection", {chi, uz, ur, R, partials, out},
                          {"char_func", "u_z", "u_r", "R", "partials", "out"}));
  const int nb = red_blocks(n);
  projection_partials_kernel<T><<<nb, RED_THREADS, 0, s>>>(rho, chi, uz, ur, R, n, partials);
  finish_kernel<<<1, RED_THREADS, 0, s>>>(partials, nb, 3, 1, 0.0, 0.0, out);
  return axi::launch_status("force_projection");
}

}  // namespace

extern "C" int64_t axi_reduction_scratch_doubles(int64_t) { return 3LL * RED_MAX_BLOCKS; }

extern "C" int axi_compute_force_on_body_f64(const double* R, const double* chi, double rho_f,
                                             double lam, const double* uz, double U, double vol,
                                             double dt, double diff, int64_t n, double* partials,
                                             double* out, void* stream) {
  axi::clear_error();
  return force_on_body<double>(R, chi, rho_f, lam, uz, U, vol, dt, diff, n, partials, out,
                               axi::as_stream(stream));
}
extern "C" int axi_compute_force_on_body_f32(const float* R, const float* chi, double rho_f,
                                             double lam, const float* uz, double U, double vol,
                                             double dt, double diff, int64_t n, double* partials,
                                             double* out, void* stream) {
  axi::clear_error();
  return force_on_body<float>(R, chi, rho_f, lam, uz, U, vol, dt, diff, n, partials, out,
                              axi::as_stream(stream));
}
extern "C" int axi_force_projection_f64(double rho, const double* chi, const double* uz,
                                        const double* ur, const double* R, int64_t n,
                                        double* partials, double* out, void* stream) {
  axi::clear_error();
  return projection<double>(rho, chi, uz, ur, R, n, partials, out, axi::as_stream(stream));
}
extern "C" int axi_force_projection_f32(double rho, const float* chi, const float* uz,
                                        const float* ur, const float* R, int64_t n,
                                        double* partials, double* out, void* stream) {
  axi::clear_error();
  return projection<float>(rho, chi, uz, ur, R, n, partials, out, axi::as_stream(stream));
}
