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
template <int N>
__device__ void dct_item_reg(const DctJob& job, int row0, bool forward, float2* dsm,
                             const float2* tw);

// Four consecutive outputs of row k (columns i .. i + 3, i a multiple of 4)
// as the TF32 pair, one float4 store each.
__device__ __forceinline__ void store_split4(const DctJob& job, int k, int i, const float (&x)[4]) {
  float hi[4], lo[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) axi_tc::tf32_split(x[q], hi[q], lo[q]);
  const long long o = (long long)k * job.rows + i;
  *reinterpret_cast<float4*>(job.out_hi + o) = make_float4(hi[0], hi[1], hi[2], hi[3]);
  *reinterpret_cast<float4*>(job.out_lo + o) = make_float4(lo[0], lo[1], lo[2], lo[3]);
}

// Residual of the refinement, x = in - (A psi) / r at (row i, column j):
//   (A psi) / r = [(c - W) + (c - E) + (c - S) + (c - N)] / (r dx^2)
//                 + (N - S) / (2 dx r^2)
// with the operator's boundary rows: W := c at j = 0 and E := c at j = N - 1
// (Neumann z ends), S := 0 below the axis row, N := c above the outer row
// and no first-derivative term there (its row of the r operator is
// (psi_{nr-1} - psi_{nr-2}) / dx^2 only). psi is the pair psi + psi_lo:
// each neighbour difference is the difference of the high parts (exact for
// close values) plus that of the low parts, so the residual sees psi to the
// pair's precision, not to its float rounding.
struct PsiPair {
  float h, l;
};
__device__ __forceinline__ float pdiff(PsiPair a, PsiPair b) { return (a.h - b.h) + (a.l - b.l); }
__device__ __forceinline__ float residual_value(float in, PsiPair c, PsiPair w, PsiPair e,
                                                PsiPair s, PsiPair n, float k1, float k2) {
  return in - ((pdiff(c, w) + pdiff(c, e)) + (pdiff(c, s) + pdiff(c, n))) * k1 +
         pdiff(s, n) * k2;
}

__device__ __forceinline__ float residual_at(const DctJob& job, int i, int j) {
  const int N = job.N, nr = job.rows;
  const long long o = (long long)i * N + j;
  const float* ph = job.psi + o;
  const float* pl = job.psi_lo + o;
  const PsiPair c{ph[0], pl[0]};
  const PsiPair w = j > 0 ? PsiPair{ph[-1], pl[-1]} : c;
  const PsiPair e = j + 1 < N ? PsiPair{ph[1], pl[1]} : c;
  const PsiPair s = i > 0 ? PsiPair{ph[-N], pl[-N]} : PsiPair{0.0f, 0.0f};
  const PsiPair n = i + 1 < nr ? PsiPair{ph[N], pl[N]} : c;
  const float k1 = job.two_over_dx * job.rinv2dx[i];
  const float k2 = i + 1 < nr ? job.inv_2dx * job.rinv2[i] : 0.0f;
  return residual_value(job.in[o], c, w, e, s, n, k1, k2);
}

// Forward input element (row i, column j): the field, or the refinement residual.
__device__ __forceinline__ float forward_input(const DctJob& job, int i, int j) {
  return job.psi ? residual_at(job, i, j) : job.in[(long long)i * job.N + j];
}

// Bulk prefetch of `bytes` (a multiple of 16, 16-byte aligned) into L2.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

__global__ void __launch_bounds__(THREADS) dct_rows_kernel(const DctJob* __restrict__ jobs,
                                                           const int4* __restrict__ items,
                                                           int n_items, int ahead, int forward) {
  extern __shared__ __align__(16) float2 dsm[];
  float2* a = dsm;
  float2* b = dsm + ELEMS;
  __shared__ DctJob sjob;
  const int4 it = items[blockIdx.x];
  if (threadIdx.x == 0) sjob = jobs[it.x];
  if (threadIdx.x == 32 && blockIdx.x + ahead < n_items) {
    // the rows of the item one resident wave ahead (`ahead` blocks fit on
    // the GPU at once), fetched into L2 while this item is transformed: the
    // block that takes it finds its rows there instead of in DRAM. Rows of
    // an item are contiguous.
    const int4 nx = items[blockIdx.x + ahead];
    const DctJob& nj = jobs[nx.x];
    const int nrows = min(rows_for(nj.N), nj.rows - nx.y);
    const uint32_t bytes = (uint32_t)nrows * (uint32_t)nj.N * 4u;
    const long long off = (long long)nx.y * nj.N;
    prefetch_l2(nj.in + off, bytes);
    if (!forward && nj.row_scale) prefetch_l2(nj.row_scale + off, bytes);
    if (forward && nj.psi) {
      prefetch_l2(nj.psi + off, bytes);
      prefetch_l2(nj.psi_lo + off, bytes);
    }
  }
  __syncthreads();
  // the twiddle table of this row length, staged once per block at the end
  // of shared memory (every thread takes the global pointer before thread 0
  // repoints the copy)
  const float2* gtw = sjob.twiddle;
  const int n_tw = sjob.N;
  // the register path reads the table padded (reg_tw_index)
  const bool padded = reg_n1(n_tw) != 0;
  float2* tws = dsm + 3 * ELEMS - (padded ? reg_tw_size(n_tw) : n_tw);
  __syncthreads();
  if (threadIdx.x == 0) sjob.twiddle = tws;
  for (int m = threadIdx.x; m < n_tw; m += blockDim.x)
    tws[padded ? reg_tw_index(m) : m] = __ldg(gtw + m);
  __syncthreads();
  const DctJob& job = sjob;
  const int N = job.N, half = N / 2;
  const int row0 = it.y;
  switch (N) {
    case 256: dct_item_reg<256>(job, row0, forward != 0, dsm, tws); return;
    case 512: dct_item_reg<512>(job, row0, forward != 0, dsm, tws); return;
    case 768: dct_item_reg<768>(job, row0, forward != 0, dsm, tws); return;
    case 1024: dct_item_reg<1024>(job, row0, forward != 0, dsm, tws); return;
    case 1536: dct_item_fixed<1536>(job, row0, forward != 0, a, b); return;
    case 2048: dct_item_fixed<2048>(job, row0, forward != 0, a, b); return;
    default: break;
  }
  const int nrows = min(rows_per_item(N), job.rows - row0);
  if (forward) {
    // v[n] = x[2n], v[N-1-n] = x[2n+1]
    for (int t = threadIdx.x; t < nrows * N; t += blockDim.x) {
      const int r = t / N, p = t - r * N;
      const float x = forward_input(job, row0 + r, p);
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
      const long long g = (long long)(row0 + r) * N + k;
      float y = job.in[g];
      if (job.row_scale) y = y * job.row_scale[g];
      xs[r * N + k] = y * job.scale[k];
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
      const float x = r < nrows ? forward_input(job, row0 + r, p) : 0.0f;
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
      const long long g = (long long)(row0 + r) * N + k;
      float y = r < nrows ? job.in[g] : 0.0f;
      if (job.row_scale && r < nrows) y = y * job.row_scale[g];
      xs[r * N + k] = y * job.scale[k];
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

// ---------------------------------------------------------------------------
// Register-resident FFT: decimation in frequency over a register array with
// compile-time indices (radix 3 first, then 2). Output position p holds
// X[dif_index(L, p)].
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int dif_radix(int L) { return (L % 3 == 0) ? 3 : 2; }
__host__ __device__ constexpr int dif_index(int L, int p) {
  return L == 1 ? 0
                : (p / (L / dif_radix(L))) +
                      dif_radix(L) * dif_index(L / dif_radix(L), p % (L / dif_radix(L)));
}

// dif_index(L, p) for all p, evaluated at compile time.
template <int L>
struct DifPerm {
  int v[L];
  __host__ __device__ constexpr DifPerm() : v() {
    for (int p = 0; p < L; ++p) v[p] = dif_index(L, p);
  }
};

// Sub-transform of length L at offset OFF of the register array v (size TOT);
// tw: exp(-2 pi i m / NT), m < NT, in shared memory at reg_tw_index(m).
template <int TOT, int L, int OFF, int NT, bool FWD>
__device__ __forceinline__ void dif_rec(float2 (&v)[TOT], const float2* tw) {
  if constexpr (L > 1) {
    constexpr int R = dif_radix(L);
    constexpr int L1 = L / R;
#pragma unroll
    for (int j = 0; j < L1; ++j) {
      float2 o[R];
      if constexpr (R == 2) {
        const float2 a0 = v[OFF + j], a1 = v[OFF + j + L1];
        o[0] = cadd(a0, a1);
        o[1] = csub(a0, a1);
      } else {
        const float h = 0.86602540378443864676f;
        const float2 a0 = v[OFF + j], a1 = v[OFF + j + L1], a2 = v[OFF + j + 2 * L1];
        const float2 t1 = cadd(a1, a2), t2 = csub(a1, a2);
        const float2 m = make_float2(a0.x - 0.5f * t1.x, a0.y - 0.5f * t1.y);
        const float2 r = FWD ? make_float2(h * t2.y, -h * t2.x) : make_float2(-h * t2.y, h * t2.x);
        o[0] = cadd(a0, t1);
        o[1] = cadd(m, r);
        o[2] = csub(m, r);
      }
      v[OFF + j] = o[0];
#pragma unroll
      for (int q = 1; q < R; ++q) {
        if (j == 0) {
          v[OFF + j + q * L1] = o[q];
        } else {
          float2 w = tw[reg_tw_index(j * q * (NT / L))];
          if (!FWD) w = conj2(w);
          v[OFF + j + q * L1] = cmul(o[q], w);
        }
      }
    }
    dif_rec<TOT, L1, OFF, NT, FWD>(v, tw);
    dif_rec<TOT, L1, OFF + L1, NT, FWD>(v, tw);
    if constexpr (R == 3) dif_rec<TOT, L1, OFF + 2 * L1, NT, FWD>(v, tw);
  }
}

// Four-step FFT of one complex row of length N = N1 x N2 held by one warp in
// `buf` (N + N1 complex values): input in natural order, output in natural
// order (in buf[0, N)). x[N2 n1 + n2] -> X[k1 + N1 k2]. With N1, N2 <= 32
// every lane has at most one transform per pass; all lanes reach every
// __syncwarp.
template <int N, int N1, bool FWD>
__device__ __forceinline__ void warp_fft(float2* buf, const float2* tw, int lane) {
  constexpr int N2 = N / N1;
  constexpr int P = N2 + 1;  // padded row stride between the passes
  static_assert(N1 <= 32 && N2 <= 32 && N1 * N2 == N, "four-step split");
  constexpr DifPerm<N1> perm1{};
  constexpr DifPerm<N2> perm2{};
  // pass 1: the length-N1 transform over n1 for n2 = lane
  const int n2 = lane;
  float2 v[N1];
  if (n2 < N2) {
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) v[n1] = buf[N2 * n1 + n2];
    dif_rec<N1, N1, 0, N, FWD>(v, tw);
  }
  __syncwarp();
  if (n2 < N2) {
    // twiddle exp(-+2 pi i n2 k1 / N), stored as [k1][n2]
#pragma unroll
    for (int p = 0; p < N1; ++p) {
      const int k1 = perm1.v[p];
      float2 w = tw[reg_tw_index(n2 * k1)];
      if (!FWD) w = conj2(w);
      buf[k1 * P + n2] = n2 == 0 ? v[p] : cmul(v[p], w);
    }
  }
  __syncwarp();
  // pass 2: the length-N2 transform over n2 for k1 = lane
  const int k1 = lane;
  float2 o[N2];
  if (k1 < N1) {
#pragma unroll
    for (int m = 0; m < N2; ++m) o[m] = buf[k1 * P + m];
    dif_rec<N2, N2, 0, N, FWD>(o, tw);
  }
  __syncwarp();
  if (k1 < N1) {
#pragma unroll
    for (int p = 0; p < N2; ++p) buf[k1 + N1 * perm2.v[p]] = o[p];
  }
  __syncwarp();
}

// Z = V_a + i V_b for two real rows packed as (a, b): V[k] = exp(i pi k / 2N)
// (X[k] - i X[N-k]) per row, x = X[k], y = X[N-k].
__device__ __forceinline__ float2 inverse_pre(float2 cs, float2 x, float2 y) {
  const float2 va = make_float2(cs.x * x.x + cs.y * y.x, cs.y * x.x - cs.x * y.x);
  const float2 vb = make_float2(cs.x * x.y + cs.y * y.y, cs.y * x.y - cs.x * y.y);
  return make_float2(va.x - vb.y, va.y + vb.x);
}

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }

// Four consecutive columns (float4 group at column p) of one row of the psi pair.
struct Pair4 {
  float4 h, l;
};
__device__ __forceinline__ Pair4 ld_pair4(const DctJob& job, long long o) {
  return Pair4{ld4(job.psi + o), ld4(job.psi_lo + o)};
}
__device__ __forceinline__ PsiPair ld_pair(const DctJob& job, long long o) {
  return PsiPair{job.psi[o], job.psi_lo[o]};
}
__device__ __forceinline__ PsiPair pick(const Pair4& a, int q) {
  return q == 0 ? PsiPair{a.h.x, a.l.x}
                : q == 1 ? PsiPair{a.h.y, a.l.y} : q == 2 ? PsiPair{a.h.z, a.l.z}
                                                            : PsiPair{a.h.w, a.l.w};
}

// residual_value on four consecutive columns of one row: c the row's psi,
// w / e the values left of column 0 / right of column 3 of the group, s / n
// the rows below / above.
__device__ __forceinline__ float4 residual4(float4 in, const Pair4& c, PsiPair w, PsiPair e,
                                            const Pair4& s, const Pair4& n, float k1, float k2) {
  return make_float4(
      residual_value(in.x, pick(c, 0), w, pick(c, 1), pick(s, 0), pick(n, 0), k1, k2),
      residual_value(in.y, pick(c, 1), pick(c, 0), pick(c, 2), pick(s, 1), pick(n, 1), k1, k2),
      residual_value(in.z, pick(c, 2), pick(c, 1), pick(c, 3), pick(s, 2), pick(n, 2), k1, k2),
      residual_value(in.w, pick(c, 3), pick(c, 2), e, pick(s, 3), pick(n, 3), k1, k2));
}

// Residual rows ga, ga + 1 (global) of the refinement into one warp buffer
// as z[n] = x_a[n] + i x_b[n] in Makhoul order, as the plain forward path
// stores the field rows. Rows missing from the item are zero.
template <int N>
__device__ __forceinline__ void residual_pair_to_buf(const DctJob& job, int ga, bool has_a,
                                                     bool has_b, int lane, float2* buf) {
  constexpr int NV = N / 128;  // float4 groups per lane and row
  const int nr = job.rows, gb = ga + 1;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  const long long oa = (long long)ga * N, ob = oa + N;
  const float k1a = has_a ? job.two_over_dx * job.rinv2dx[ga] : 0.0f;
  const float k2a = has_a ? job.inv_2dx * job.rinv2[ga] : 0.0f;
  const float k1b = has_b ? job.two_over_dx * job.rinv2dx[gb] : 0.0f;
  const float k2b = (has_b && gb + 1 < nr) ? job.inv_2dx * job.rinv2[gb] : 0.0f;
  // two float4 groups per iteration: the loads of the second are in flight
  // while the first is formed (0.247 -> 0.239 ms for the two transforms;
  // four groups were no faster)
#pragma unroll 2
  for (int m = 0; m < NV; ++m) {
    const int p = 4 * (lane + 32 * m);
    float4 xa = zero, xb = zero;
    if (has_a) {
      const Pair4 ca = ld_pair4(job, oa + p);
      const Pair4 sa = ga > 0 ? ld_pair4(job, oa - N + p) : Pair4{zero, zero};
      // row a is never the outer row (rows come in even-aligned pairs)
      const Pair4 cb = has_b ? ld_pair4(job, ob + p) : ca;
      const PsiPair wa = p > 0 ? ld_pair(job, oa + p - 1) : pick(ca, 0);
      const PsiPair ea = p + 4 < N ? ld_pair(job, oa + p + 4) : pick(ca, 3);
      xa = residual4(ld4(job.in + oa + p), ca, wa, ea, sa, cb, k1a, k2a);
      if (has_b) {
        const Pair4 nb = gb + 1 < nr ? ld_pair4(job, ob + N + p) : cb;
        const PsiPair wb = p > 0 ? ld_pair(job, ob + p - 1) : pick(cb, 0);
        const PsiPair eb = p + 4 < N ? ld_pair(job, ob + p + 4) : pick(cb, 3);
        xb = residual4(ld4(job.in + ob + p), cb, wb, eb, ca, nb, k1b, k2b);
      }
    }
    const int h = p >> 1;
    *reinterpret_cast<float4*>(buf + h) = make_float4(xa.x, xb.x, xa.z, xb.z);
    *reinterpret_cast<float4*>(buf + N - 2 - h) = make_float4(xa.w, xb.w, xa.y, xb.y);
  }
}

// Work item of the register path: warp w transforms real rows 2w, 2w + 1 of
// the item as one complex row in its own buffer; the block then stores the
// results transposed (rows fastest).
template <int N>
__device__ void dct_item_reg(const DctJob& job, int row0, bool forward, float2* dsm,
                             const float2* tw) {
  constexpr int N1 = reg_n1(N);
  constexpr int W = reg_warps(N);
  constexpr int BUF = reg_buf(N);
  static_assert(BUF >= N + N1 - 1 && BUF % 16 == 2, "warp buffer stride");
  constexpr int RR = 2 * W;  // real rows of a full item
  static_assert(RR % 4 == 0, "float4 output groups");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nrows = min(2 * W, job.rows - row0);  // real rows of this item
  const int ra = 2 * warp, rb = ra + 1;
  if (warp < W && forward && job.psi) {
    // refinement: the residual rows of the pair, four columns per lane and
    // float4 group at a time, straight into the warp buffer (Makhoul order)
    float2* buf = dsm + warp * BUF;
    residual_pair_to_buf<N>(job, row0 + ra, ra < nrows, rb < nrows, lane, buf);
    __syncwarp();
    warp_fft<N, N1, true>(buf, tw, lane);
  } else if (warp < W) {
    float2* buf = dsm + warp * BUF;
    const bool has_a = ra < nrows, has_b = rb < nrows;
    const float* ia = job.in + (long long)(row0 + ra) * N;
    const float* ib = job.in + (long long)(row0 + rb) * N;
    // rows are read as float4 (N a multiple of 4, rows 16-byte aligned), all
    // loads of a lane issued before their first use
    constexpr int NV = N / 128;  // float4 per lane per row
    const float4* va4 = reinterpret_cast<const float4*>(ia);
    const float4* vb4 = reinterpret_cast<const float4*>(ib);
    float4 xa[NV], xb[NV];
#pragma unroll
    for (int m = 0; m < NV; ++m) {
      xa[m] = has_a ? va4[lane + 32 * m] : make_float4(0.f, 0.f, 0.f, 0.f);
      xb[m] = has_b ? vb4[lane + 32 * m] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (forward) {
      // z[n] = v_a[n] + i v_b[n], v[n] = x[2n], v[N-1-n] = x[2n+1]
      // (h, h + 1) and (N - 2 - h, N - 1 - h) are 16-byte aligned pairs (h
      // even, buffers 16-byte aligned): one float4 store each
#pragma unroll
      for (int m = 0; m < NV; ++m) {
        const int p = 4 * (lane + 32 * m);  // even
        const int h = p >> 1;
        *reinterpret_cast<float4*>(buf + h) = make_float4(xa[m].x, xb[m].x, xa[m].z, xb[m].z);
        *reinterpret_cast<float4*>(buf + N - 2 - h) =
            make_float4(xa[m].w, xb[m].w, xa[m].y, xb[m].y);
      }
      __syncwarp();
      warp_fft<N, N1, true>(buf, tw, lane);
    } else {
      // X = Y / c_k; Z[k] = V_a[k] + i V_b[k], V[k] = exp(i pi k / 2N) (X[k] - i X[N-k])
      const float4* sc4 = reinterpret_cast<const float4*>(job.scale);
      if (job.row_scale) {
        // Y = G .* inv_eig, elementwise, before 1 / c_k
        const float4* ra4 = reinterpret_cast<const float4*>(job.row_scale + (long long)(row0 + ra) * N);
        const float4* rb4 = reinterpret_cast<const float4*>(job.row_scale + (long long)(row0 + rb) * N);
#pragma unroll
        for (int m = 0; m < NV; ++m) {
          const float4 sa = has_a ? __ldg(ra4 + lane + 32 * m) : make_float4(0.f, 0.f, 0.f, 0.f);
          const float4 sb = has_b ? __ldg(rb4 + lane + 32 * m) : make_float4(0.f, 0.f, 0.f, 0.f);
          xa[m] = make_float4(xa[m].x * sa.x, xa[m].y * sa.y, xa[m].z * sa.z, xa[m].w * sa.w);
          xb[m] = make_float4(xb[m].x * sb.x, xb[m].y * sb.y, xb[m].z * sb.z, xb[m].w * sb.w);
        }
      }
#pragma unroll
      for (int m = 0; m < NV; ++m) {
        const float4 sc = __ldg(sc4 + lane + 32 * m);
        const int k = 4 * (lane + 32 * m);
        *reinterpret_cast<float4*>(buf + k) =
            make_float4(xa[m].x * sc.x, xb[m].x * sc.x, xa[m].y * sc.y, xb[m].y * sc.y);
        *reinterpret_cast<float4*>(buf + k + 2) =
            make_float4(xa[m].z * sc.z, xb[m].z * sc.z, xa[m].w * sc.w, xb[m].w * sc.w);
      }
      __syncwarp();
      // Z[k] and Z[N-k] both depend on X[k] and X[N-k] only: each lane
      // rewrites its own pairs in place
      // (unrolled by 4 so the rotation-table loads of several k are in flight
      // together)
      const float2* __restrict__ rot = job.rot;
#pragma unroll 4
      for (int k = lane; k <= N / 2; k += 32) {
        const float2 rk = __ldg(rot + k), rn = __ldg(rot + (N - k) % N);
        const float2 xk = buf[k];
        const float2 xn = k == 0 ? make_float2(0.0f, 0.0f) : buf[N - k];
        const float2 zk = inverse_pre(rk, xk, xn);
        if (k != 0 && k != N / 2) buf[N - k] = inverse_pre(rn, xn, xk);
        buf[k] = zk;
      }
      __syncwarp();
      warp_fft<N, N1, false>(buf, tw, lane);
    }
  }
  __syncthreads();
  // transposed stores, four consecutive rows per thread as float4 (rows is a
  // multiple of 4 and items start at multiples of RR, so both the row count
  // of an item and the output offsets are multiples of 4)
  constexpr int G = RR / 4;
  if (forward) {
#pragma unroll 4
    for (int t = threadIdx.x; t < G * N; t += blockDim.x) {
      const int k = t / G, g = t - k * G;
      const int r0 = 4 * g;
      if (r0 >= nrows) continue;
      const float2 cs = job.rot[k];
      const float sk = job.scale[k];
      float x[4];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float2* z = dsm + (2 * g + h) * BUF;
        const float2 zk = z[k], zn = z[k == 0 ? 0 : N - k];
        // V_a = (Z[k] + conj Z[N-k]) / 2, V_b = (Z[k] - conj Z[N-k]) / 2i
        const float2 va = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
        const float2 vb = make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x));
        x[2 * h] = sk * (va.x * cs.x + va.y * cs.y);
        x[2 * h + 1] = sk * (vb.x * cs.x + vb.y * cs.y);
      }
      store_split4(job, k, row0 + r0, x);
    }
  } else {
    const float inv_n = 1.0f / (float)N;
#pragma unroll 4
    for (int t = threadIdx.x; t < G * N; t += blockDim.x) {
      const int j = t / G, g = t - j * G;
      const int r0 = 4 * g;
      if (r0 >= nrows) continue;
      const int src = (j & 1) ? N - 1 - (j >> 1) : (j >> 1);
      const float2 z0 = dsm[(2 * g) * BUF + src], z1 = dsm[(2 * g + 1) * BUF + src];
      float x[4] = {z0.x * inv_n, z0.y * inv_n, z1.x * inv_n, z1.y * inv_n};
      store_split4(job, j, row0 + r0, x);
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

int launch(const DctJob* jobs_dev, const int4* items_dev, int n_items, bool forward,
           cudaStream_t s, int prefetch_waves) {
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
  static int per_sm = 0;
  if (per_sm == 0) {
    int b = 0;
    per_sm = (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, dct_rows_kernel, THREADS,
                                                           SMEM_BYTES) == cudaSuccess && b > 0)
                 ? b
                 : 1;
  }
  // prefetch distance: `prefetch_waves` resident waves ahead (n_items: none)
  const int wave = per_sm * axi::sm_count();
  const int ahead = prefetch_waves < 0 ? n_items : wave * (prefetch_waves > 0 ? prefetch_waves : 1);
  dct_rows_kernel<<<n_items, THREADS, SMEM_BYTES, s>>>(jobs_dev, items_dev, n_items, ahead,
                                                       forward ? 1 : 0);
  return axi::launch_status("dct_rows");
}

}  // namespace axi_dct
