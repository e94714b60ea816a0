// Grouped orthonormal DCT-II / DCT-III along rows in double (see dct64.cuh).
#include <cstring>
#include <mutex>
#include <vector>

#include "dct64.cuh"

namespace axi_dct64 {
namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) {
  return make_double2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ double2 conj2(double2 a) { return make_double2(a.x, -a.y); }

// One Stockham stage of radix R on `nrows` rows of length N; forward uses
// exp(-2 pi i / N), inverse its conjugate (no 1/N).
template <int R>
__device__ void stage(const double2* __restrict__ src, double2* __restrict__ dst, int N,
                      int nrows, int Ns, const double2* __restrict__ tw, bool forward) {
  const int per_row = N / R;
  const int tstride = N / (Ns * R);
  for (int t = threadIdx.x; t < per_row * nrows; t += blockDim.x) {
    const int row = t / per_row, j = t - row * per_row;
    const double2* x = src + row * N;
    double2* y = dst + row * N;
    const int k = j % Ns;
    double2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      v[q] = x[j + q * per_row];
      if (q > 0) {
        double2 w = tw[(k * q * tstride) % N];
        if (!forward) w = conj2(w);
        v[q] = cmul(v[q], w);
      }
    }
    double2 o[R];
    if constexpr (R == 2) {
      o[0] = cadd(v[0], v[1]);
      o[1] = csub(v[0], v[1]);
    } else if constexpr (R == 4) {
      const double2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
      const double2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
      const double2 r = forward ? make_double2(d13.y, -d13.x) : make_double2(-d13.y, d13.x);
      o[0] = cadd(s02, s13);
      o[1] = cadd(d02, r);
      o[2] = csub(s02, s13);
      o[3] = csub(d02, r);
    } else {  // R == 3
      const double h = 0.86602540378443864676;  // sqrt(3) / 2
      const double2 t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
      const double2 m = make_double2(v[0].x - 0.5 * t1.x, v[0].y - 0.5 * t1.y);
      const double2 r =
          forward ? make_double2(h * t2.y, -h * t2.x) : make_double2(-h * t2.y, h * t2.x);
      o[0] = cadd(v[0], t1);
      o[1] = cadd(m, r);
      o[2] = csub(m, r);
    }
    const int base = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int s = 0; s < R; ++s) y[base + s * Ns] = o[s];
  }
}

__device__ void fft_rows(double2*& a, double2*& b, const Job& job, const double2* tw, int nrows,
                         bool forward) {
  int Ns = 1;
  for (int st = 0; st < job.nstages; ++st) {
    const int R = job.radix[st];
    if (R == 4)
      stage<4>(a, b, job.N, nrows, Ns, tw, forward);
    else if (R == 2)
      stage<2>(a, b, job.N, nrows, Ns, tw, forward);
    else
      stage<3>(a, b, job.N, nrows, Ns, tw, forward);
    __syncthreads();
    double2* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
}

__global__ void __launch_bounds__(THREADS) dct64_rows_kernel(const Job* __restrict__ jobs,
                                                             const int4* __restrict__ items,
                                                             int forward) {
  extern __shared__ __align__(16) double2 sm[];
  double2* a = sm;
  double2* b = sm + ELEMS;
  double2* tw = sm + 2 * ELEMS;
  __shared__ Job job;
  const int4 it = items[blockIdx.x];
  if (threadIdx.x == 0) job = jobs[it.x];
  __syncthreads();
  const int N = job.N;
  for (int m = threadIdx.x; m < N; m += blockDim.x) tw[m] = job.twiddle[m];
  const int row0 = it.y;
  const int nrows = min(rows_per_item(N), job.rows - row0);
  if (forward) {
    // v[n] = x[2n], v[N-1-n] = x[2n+1]
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int r = t / N, p = t - r * N;
      const double x = job.in[(long long)(row0 + r) * N + p];
      const int d = (p & 1) ? N - 1 - (p >> 1) : (p >> 1);
      a[r * N + d] = make_double2(x, 0.0);
    }
    __syncthreads();
    fft_rows(a, b, job, tw, nrows, true);
    // X[k] = c_k Re(exp(-i pi k / 2N) V[k]), row-major
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int r = t / N, k = t - r * N;
      const double2 V = a[r * N + k];
      const double2 cs = job.rot[k];
      job.out[(long long)(row0 + r) * N + k] = job.scale[k] * (V.x * cs.x + V.y * cs.y);
    }
  } else {
    // X[k] = Y[k] / c_k; V[k] = exp(i pi k / 2N) (X[k] - i X[N-k]), X[N] = 0
    double* xs = reinterpret_cast<double*>(b);
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int r = t / N, k = t - r * N;
      xs[r * N + k] = job.in[(long long)(row0 + r) * N + k] * job.scale[k];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int r = t / N, k = t - r * N;
      const double xk = xs[r * N + k];
      const double xn = k == 0 ? 0.0 : xs[r * N + N - k];
      const double2 cs = job.rot[k];
      a[r * N + k] = make_double2(cs.x * xk + cs.y * xn, cs.y * xk - cs.x * xn);
    }
    __syncthreads();
    fft_rows(a, b, job, tw, nrows, false);
    // y[2n] = Re v[n] / N, y[2n+1] = Re v[N-1-n] / N, row-major
    const double inv_n = 1.0 / (double)N;
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int r = t / N, j = t - r * N;
      const int src = (j & 1) ? N - 1 - (j >> 1) : (j >> 1);
      job.out[(long long)(row0 + r) * N + j] = a[r * N + src].x * inv_n;
    }
  }
}

}  // namespace

bool plan_radices(int N, int* radix, int* nstages) {
  if (N < 2 || (N & 1) || N > ELEMS) return false;
  int n = N, s = 0;
  while (n % 4 == 0 && s < MAX_STAGES) { radix[s++] = 4; n /= 4; }
  while (n % 2 == 0 && s < MAX_STAGES) { radix[s++] = 2; n /= 2; }
  while (n % 3 == 0 && s < MAX_STAGES) { radix[s++] = 3; n /= 3; }
  *nstages = s;
  return n == 1;
}

int launch(const Job* jobs_dev, const int4* items_dev, int n_items, bool forward,
           cudaStream_t s) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(dct64_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                SMEM_BYTES);
  });
  if (attr != cudaSuccess) {
    axi::set_error("dct64: cannot reserve %d bytes of shared memory", SMEM_BYTES);
    return AXI_ERR_CUDA;
  }
  if (n_items <= 0) return AXI_OK;
  dct64_rows_kernel<<<n_items, THREADS, SMEM_BYTES, s>>>(jobs_dev, items_dev, forward ? 1 : 0);
  return axi::launch_status("dct64_rows");
}

}  // namespace axi_dct64

// ---------------------------------------------------------------------------
// Standalone FP64 row transforms for callers outside the rigid engine's plan
// (the soft-sphere engine's spectral solve). A plan is one device buffer: the
// Job record, then one work item per group of rows; it fixes the input and
// output arrays, so a step can launch it with no host data (and inside a CUDA
// graph). Tables: the double layout of the engine's dct_table (twiddles,
// rotations, c_k, 1 / c_k).
// ---------------------------------------------------------------------------
namespace {
constexpr size_t JOB_BYTES = (sizeof(axi_dct64::Job) + 15) & ~size_t(15);
inline int items_of(int rows, int N) {
  const int r = axi_dct64::rows_per_item(N);
  return (rows + r - 1) / r;
}
}  // namespace

extern "C" int64_t axi_dct64_plan_bytes(int rows, int N) {
  if (rows < 1 || N < 2) return 0;
  return (int64_t)(JOB_BYTES + (size_t)items_of(rows, N) * sizeof(int4));
}

extern "C" int axi_dct64_plan_f64(const double* in, double* out, int rows, int N,
                                  const double* table, int forward, void* plan_dev,
                                  void* stream) {
  axi::clear_error();
  const char* what = "dct64_plan";
  AXI_TRY(axi::check_ptr(what, in, "in"));
  AXI_TRY(axi::check_ptr(what, out, "out"));
  AXI_TRY(axi::check_ptr(what, table, "table"));
  AXI_TRY(axi::check_ptr(what, plan_dev, "plan"));
  axi_dct64::Job j;
  memset(&j, 0, sizeof(j));
  if (rows < 1 || !axi_dct64::plan_radices(N, j.radix, &j.nstages)) {
    axi::set_error("%s: %d rows of length %d have no double DCT plan (N even, factors 2 and 3 "
                   "only, <= %d)", what, rows, N, axi_dct64::ELEMS);
    return AXI_ERR_INVALID;
  }
  j.N = N;
  j.rows = rows;
  j.in = in;
  j.out = out;
  j.twiddle = reinterpret_cast<const double2*>(table);
  j.rot = reinterpret_cast<const double2*>(table + (size_t)2 * N);
  j.scale = table + (size_t)(forward ? 4 : 5) * N;
  const int n_items = items_of(rows, N);
  std::vector<unsigned char> buf(JOB_BYTES + (size_t)n_items * sizeof(int4), 0);
  memcpy(buf.data(), &j, sizeof(j));
  int4* items = reinterpret_cast<int4*>(buf.data() + JOB_BYTES);
  const int r = axi_dct64::rows_per_item(N);
  for (int q = 0; q < n_items; ++q) items[q] = make_int4(0, q * r, 0, 0);
  cudaStream_t s = axi::as_stream(stream);
  if (cudaMemcpyAsync(plan_dev, buf.data(), buf.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return axi::launch_status(what);
  return AXI_OK;
}

extern "C" int axi_dct64_run_f64(const void* plan_dev, int rows, int N, int forward,
                                 void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("dct64_run", plan_dev, "plan"));
  if (rows < 1 || N < 2) {
    axi::set_error("dct64_run: invalid size %d x %d", rows, N);
    return AXI_ERR_INVALID;
  }
  const unsigned char* base = static_cast<const unsigned char*>(plan_dev);
  return axi_dct64::launch(reinterpret_cast<const axi_dct64::Job*>(base),
                           reinterpret_cast<const int4*>(base + JOB_BYTES), items_of(rows, N),
                           forward != 0, axi::as_stream(stream));
}
