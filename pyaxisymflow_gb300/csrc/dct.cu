// Grouped orthonormal DCT-II / DCT-III along rows (see dct.cuh).
#include <mutex>

#include "dct.cuh"
#include "tc_gemm.cuh"

namespace axi_dct {
namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 conj2(float2 a) { return make_float2(a.x, -a.y); }

// One Stockham stage of radix R on `nrows` rows of length N (row stride N in
// both buffers). Forward transforms use exp(-2 pi i / N); inverse ones the
// conjugate (no 1/N).
template <int R>
__device__ void stockham_stage(const float2* __restrict__ src, float2* __restrict__ dst, int N,
                               int nrows, int Ns, const float2* __restrict__ tw, bool forward) {
  const int per_row = N / R;
  const int tstride = N / (Ns * R);  // twiddle index step
  for (int t = threadIdx.x; t < per_row * nrows; t += blockDim.x) {
    const int row = t / per_row, j = t - row * per_row;
    const float2* x = src + row * N;
    float2* y = dst + row * N;
    const int k = j % Ns;
    float2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      v[q] = x[j + q * per_row];
      if (q > 0) {
        float2 w = tw[(k * q * tstride) % N];
        if (!forward) w = conj2(w);
        v[q] = cmul(v[q], w);
      }
    }
    float2 o[R];
    if constexpr (R == 2) {
      o[0] = cadd(v[0], v[1]);
      o[1] = csub(v[0], v[1]);
    } else if constexpr (R == 4) {
      const float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
      const float2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
      // -i * d13 (forward) or +i * d13 (inverse)
      const float2 rot = forward ? make_float2(d13.y, -d13.x) : make_float2(-d13.y, d13.x);
      o[0] = cadd(s02, s13);
      o[1] = cadd(d02, rot);
      o[2] = csub(s02, s13);
      o[3] = csub(d02, rot);
    } else {  // R == 3
      const float h = 0.86602540378443864676f;  // sqrt(3) / 2
      const float2 t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
      const float2 m = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
      // -i h t2 (forward) or +i h t2 (inverse)
      const float2 r = forward ? make_float2(h * t2.y, -h * t2.x) : make_float2(-h * t2.y, h * t2.x);
      o[0] = cadd(v[0], t1);
      o[1] = cadd(m, r);
      o[2] = csub(m, r);
    }
    const int base = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int s = 0; s < R; ++s) y[base + s * Ns] = o[s];
  }
}

__device__ void fft_rows(float2*& a, float2*& b, const DctJob& job, int nrows, bool forward) {
  int Ns = 1;
  for (int st = 0; st < job.nstages; ++st) {
    const int R = job.radix[st];
    if (R == 4)
      stockham_stage<4>(a, b, job.N, nrows, Ns, job.twiddle, forward);
    else if (R == 2)
      stockham_stage<2>(a, b, job.N, nrows, Ns, job.twiddle, forward);
    else
      stockham_stage<3>(a, b, job.N, nrows, Ns, job.twiddle, forward);
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
}

__device__ __forceinline__ void store_split(const DctJob& job, int k, int i, float v) {
  float hi, lo;
  axi_tc::tf32_split(v, hi, lo);
  const long long o = (long long)k * job.rows + i;
  job.out_hi[o] = hi;
  job.out_lo[o] = lo;
}

template <int N>
__device__ void dct_item_fixed(const DctJob& job, int row0, bool forward, float2* a, float2* b);

__global__ void __launch_bounds__(THREADS) dct_rows_kernel(const DctJob* __restrict__ jobs,
                                                           const int4* __restrict__ items,
                                                           int forward) {
  extern __shared__ __align__(16) float2 dsm[];
  float2* a = dsm;
  float2* b = dsm + ELEMS;
  float2* tws = dsm + 2 * ELEMS;
  __shared__ DctJob sjob;
  const int4 it = items[blockIdx.x];
  if (threadIdx.x == 0) sjob = jobs[it.x];
  __syncthreads();
  // the twiddle table of this row length, staged once per block (every
  // thread takes the global pointer before thread 0 repoints the copy)
  const float2* gtw = sjob.twiddle;
  const int n_tw = sjob.N;
  __syncthreads();
  if (threadIdx.x == 0) sjob.twiddle = tws;
  for (int m = threadIdx.x; m < n_tw; m += blockDim.x) tws[m] = __ldg(gtw + m);
  __syncthreads();
  const DctJob& job = sjob;
  const int N = job.N, half = N / 2;
  const int row0 = it.y;
  switch (N) {
    case 256: dct_item_fixed<256>(job, row0, forward != 0, a, b); return;
    case 512: dct_item_fixed<512>(job, row0, forward != 0, a, b); return;
    case 768: dct_item_fixed<768>(job, row0, forward != 0, a, b); return;
    case 1024: dct_item_fixed<1024>(job, row0, forward != 0, a, b); return;
    case 1536: dct_item_fixed<1536>(job, row0, forward != 0, a, b); return;
    case 2048: dct_item_fixed<2048>(job, row0, forward != 0, a, b); return;
    default: break;
  }
  const int nrows = min(rows_per_item(N), job.rows - row0);
  if (forward) {
    // v[n] = x[2n], v[N-1-n] = x[2n+1]
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int r = t / N, p = t - r * N;
      const float x = job.in[(long long)(row0 + r) * N + p];
      const int d = (p & 1) ? N - 1 - (p >> 1) : (p >> 1);
      a[r * N + d] = make_float2(x, 0.0f);
    }
    __syncthreads();
    fft_rows(a, b, job, nrows, true);
    // X[k] = c_k Re(exp(-i pi k / 2N) V[k]); written transposed, rows fastest
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int k = t / nrows, r = t - k * nrows;
      const float2 V = a[r * N + k];
      const float2 cs = job.rot[k];
      store_split(job, k, row0 + r, job.scale[k] * (V.x * cs.x + V.y * cs.y));
    }
  } else {
    // X[k] = Y[k] / c_k; V[k] = exp(i pi k / 2N) (X[k] - i X[N-k]), X[N] = 0
    float* xs = reinterpret_cast<float*>(b);
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int r = t / N, k = t - r * N;
      xs[r * N + k] = job.in[(long long)(row0 + r) * N + k] * job.scale[k];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int r = t / N, k = t - r * N;
      const float xk = xs[r * N + k];
      const float xn = k == 0 ? 0.0f : xs[r * N + N - k];
      const float2 cs = job.rot[k];
      a[r * N + k] = make_float2(cs.x * xk + cs.y * xn, cs.y * xk - cs.x * xn);
    }
    __syncthreads();
    fft_rows(a, b, job, nrows, false);
    // y[2n] = Re v[n] / N, y[2n+1] = Re v[N-1-n] / N; written transposed
    const float inv_n = 1.0f / (float)N;
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int j = t / nrows, r = t - j * nrows;
      const int src = (j & 1) ? N - 1 - (j >> 1) : (j >> 1);
      store_split(job, j, row0 + r, a[r * N + src].x * inv_n);
    }
  }
  (void)half;
}

// ---------------------------------------------------------------------------
// Specialised path for a compile-time row length N: two real rows share one
// complex FFT (real and imaginary parts), so a work item holds 2 x ELEMS / N
// real rows; all index arithmetic is constant-folded. Radices as in
// plan_radices: 4s, then a 2, then 3s.
// ---------------------------------------------------------------------------
constexpr int pow2_part(int m) { return (m % 2 == 0) ? 2 * pow2_part(m / 2) : 1; }
constexpr int radix_for(int m) { return pow2_part(m) >= 4 ? 4 : (pow2_part(m) == 2 ? 2 : 3); }

template <int N>
constexpr int packed_rows() {
  return 2 * (ELEMS / N);  // real rows per work item
}

template <int N, int NS>
__device__ __forceinline__ void fft_fixed(float2*& a, float2*& b, int ncrows,
                                          const float2* __restrict__ tw, bool forward) {
  if constexpr (NS < N) {
    constexpr int R = radix_for(N / NS);
    constexpr int per_row = N / R;
    constexpr int tstride = N / (NS * R);
    for (int t = threadIdx.x; t < per_row * ncrows; t += blockDim.x) {
      const int row = t / per_row, j = t - row * per_row;
      const float2* x = a + row * N;
      float2* y = b + row * N;
      const int k = j % NS;
      float2 v[R];
#pragma unroll
      for (int q = 0; q < R; ++q) {
        v[q] = x[j + q * per_row];
        if (q > 0 && NS > 1) {
          float2 w = tw[k * q * tstride];
          if (!forward) w = conj2(w);
          v[q] = cmul(v[q], w);
        }
      }
      float2 o[R];
      if constexpr (R == 2) {
        o[0] = cadd(v[0], v[1]);
        o[1] = csub(v[0], v[1]);
      } else if constexpr (R == 4) {
        const float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
        const float2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
        const float2 rot = forward ? make_float2(d13.y, -d13.x) : make_float2(-d13.y, d13.x);
        o[0] = cadd(s02, s13);
        o[1] = cadd(d02, rot);
        o[2] = csub(s02, s13);
        o[3] = csub(d02, rot);
      } else {
        const float h = 0.86602540378443864676f;
        const float2 t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
        const float2 m = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
        const float2 r = forward ? make_float2(h * t2.y, -h * t2.x)
                                 : make_float2(-h * t2.y, h * t2.x);
        o[0] = cadd(v[0], t1);
        o[1] = cadd(m, r);
        o[2] = csub(m, r);
      }
      const int base = (j / NS) * NS * R + k;
#pragma unroll
      for (int s = 0; s < R; ++s) y[base + s * NS] = o[s];
    }
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    fft_fixed<N, NS * R>(a, b, ncrows, tw, forward);
  }
}

template <int N>
__device__ void dct_item_fixed(const DctJob& job, int row0, bool forward, float2* a, float2* b) {
  constexpr int RR = packed_rows<N>();
  const int nrows = min(RR, job.rows - row0);   // real rows
  const int ncrows = (nrows + 1) / 2;           // complex rows
  if (forward) {
    // z[n] = v_a[n] + i v_b[n], v[n] = x[2n], v[N-1-n] = x[2n+1]
    float* af = reinterpret_cast<float*>(a);
    for (int t = threadIdx.x; t < ncrows * 2 * N; t += blockDim.x) {
      const int r = t / N, p = t - r * N;
      const float x = r < nrows ? job.in[(long long)(row0 + r) * N + p] : 0.0f;
      const int d = (p & 1) ? N - 1 - (p >> 1) : (p >> 1);
      af[2 * ((r >> 1) * N + d) + (r & 1)] = x;
    }
    __syncthreads();
    fft_fixed<N, 1>(a, b, ncrows, job.twiddle, true);
    // V_a = (Z[k] + conj Z[N-k]) / 2, V_b = (Z[k] - conj Z[N-k]) / 2i;
    // X[k] = c_k Re(exp(-i pi k / 2N) V[k]); transposed, rows fastest
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int k = t / nrows, r = t - k * nrows;
      const float2* z = a + (r >> 1) * N;
      const float2 zk = z[k], zn = z[k == 0 ? 0 : N - k];
      float2 V;
      if (r & 1)
        V = make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x));
      else
        V = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
      const float2 cs = job.rot[k];
      store_split(job, k, row0 + r, job.scale[k] * (V.x * cs.x + V.y * cs.y));
    }
  } else {
    // X = Y / c_k (staged in b); Z[k] = V_a[k] + i V_b[k],
    // V[k] = exp(i pi k / 2N) (X[k] - i X[N-k]), X[N] = 0
    float* xs = reinterpret_cast<float*>(b);
    for (int t = threadIdx.x; t < ncrows * 2 * N; t += blockDim.x) {
      const int r = t / N, k = t - r * N;
      xs[r * N + k] = r < nrows ? job.in[(long long)(row0 + r) * N + k] * job.scale[k] : 0.0f;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < ncrows * N; t += blockDim.x) {
      const int cr = t / N, k = t - cr * N;
      const float2 cs = job.rot[k];
      const float* xa = xs + (2 * cr) * N;
      const float* xb = xa + N;
      const float ak = xa[k], an = k == 0 ? 0.0f : xa[N - k];
      const float bk = xb[k], bn = k == 0 ? 0.0f : xb[N - k];
      const float2 va = make_float2(cs.x * ak + cs.y * an, cs.y * ak - cs.x * an);
      const float2 vb = make_float2(cs.x * bk + cs.y * bn, cs.y * bk - cs.x * bn);
      a[cr * N + k] = make_float2(va.x - vb.y, va.y + vb.x);
    }
    __syncthreads();
    fft_fixed<N, 1>(a, b, ncrows, job.twiddle, false);
    // y_a[j] = Re z[src] / N, y_b[j] = Im z[src] / N; transposed, rows fastest
    const float inv_n = 1.0f / (float)N;
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int j = t / nrows, r = t - j * nrows;
      const int src = (j & 1) ? N - 1 - (j >> 1) : (j >> 1);
      const float2 zv = a[(r >> 1) * N + src];
      store_split(job, j, row0 + r, ((r & 1) ? zv.y : zv.x) * inv_n);
    }
  }
}

}  // namespace

// Rows per work item: specialised lengths pack two real rows per complex row.
int rows_for(int N) {
  switch (N) {
    case 256: case 512: case 768: case 1024: case 1536: case 2048:
      return 2 * (ELEMS / N);
    default:
      return rows_per_item(N);
  }
}

bool plan_radices(int N, int* radix, int* nstages) {
  if (N < 2 || (N & 1) || N > ELEMS) return false;
  int n = N, s = 0;
  while (n % 4 == 0 && s < MAX_STAGES) { radix[s++] = 4; n /= 4; }
  while (n % 2 == 0 && s < MAX_STAGES) { radix[s++] = 2; n /= 2; }
  while (n % 3 == 0 && s < MAX_STAGES) { radix[s++] = 3; n /= 3; }
  *nstages = s;
  return n == 1;
}

int launch(const DctJob* jobs_dev, const int4* items_dev, int n_items, bool forward,
           cudaStream_t s) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(dct_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                SMEM_BYTES);
  });
  if (attr != cudaSuccess) {
    axi::set_error("dct: cannot reserve %d bytes of shared memory", SMEM_BYTES);
    return AXI_ERR_CUDA;
  }
  if (n_items <= 0) return AXI_OK;
  dct_rows_kernel<<<n_items, THREADS, SMEM_BYTES, s>>>(jobs_dev, items_dev, forward ? 1 : 0);
  return axi::launch_status("dct_rows");
}

}  // namespace axi_dct
