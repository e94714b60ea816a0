// Register-tiled SIMT GEMM template (double or float), row-major operands
// with row strides, optional elementwise epilogue scale.
//
// GB300 runs FP64 at about 1 TFLOP/s (DFMA and DMMA alike, 1/70 of its FP32
// rate), so FP64 products are bound by the FP64 pipe: each thread keeps a 4x4
// accumulator tile, operands go through shared memory in K slices, and 32x32
// block tiles give enough blocks to cover the 152 SMs on 256 x 512 fields.
#pragma once
#include "axi_common.cuh"

namespace axi_gemm {

constexpr int TM = 32;   // rows of C per block
constexpr int TN = 32;   // cols of C per block
constexpr int TK = 32;   // K slice staged in shared memory
constexpr int RM = 4;    // rows per thread
constexpr int RN = 4;    // cols per thread
constexpr int THREADS = (TM / RM) * (TN / RN);  // 64

// C[M,N] = A[M,K] B[K,N] (row strides ldc/lda/ldb), optionally .* S[M,N]
// (row stride N).
template <typename T>
__global__ void __launch_bounds__(THREADS) gemm_kernel(T* __restrict__ C, int ldc,
                                                       const T* __restrict__ A, int lda,
                                                       const T* __restrict__ B, int ldb,
                                                       const T* __restrict__ S, int M, int N,
                                                       int K) {
  __shared__ T As[TK][TM + 1];
  __shared__ T Bs[TK][TN];
  const int tx = threadIdx.x % (TN / RN);
  const int ty = threadIdx.x / (TN / RN);
  const int m0 = blockIdx.y * TM;
  const int n0 = blockIdx.x * TN;
  T acc[RM][RN];
#pragma unroll
  for (int a = 0; a < RM; ++a)
#pragma unroll
    for (int b = 0; b < RN; ++b) acc[a][b] = T(0);

  for (int k0 = 0; k0 < K; k0 += TK) {
    for (int e = threadIdx.x; e < TM * TK; e += THREADS) {
      const int r = e / TK, kk = e % TK;
      const int gm = m0 + r, gk = k0 + kk;
      As[kk][r] = (gm < M && gk < K) ? A[(long long)gm * lda + gk] : T(0);
    }
    for (int e = threadIdx.x; e < TK * TN; e += THREADS) {
      const int kk = e / TN, cidx = e % TN;
      const int gk = k0 + kk, gn = n0 + cidx;
      Bs[kk][cidx] = (gk < K && gn < N) ? B[(long long)gk * ldb + gn] : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < TK; ++kk) {
      T a[RM], b[RN];
#pragma unroll
      for (int q = 0; q < RM; ++q) a[q] = As[kk][ty * RM + q];
#pragma unroll
      for (int q = 0; q < RN; ++q) b[q] = Bs[kk][tx + q * (TN / RN)];
#pragma unroll
      for (int p = 0; p < RM; ++p)
#pragma unroll
        for (int q = 0; q < RN; ++q) acc[p][q] = fma(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < RM; ++p) {
    const int gm = m0 + ty * RM + p;
    if (gm >= M) continue;
#pragma unroll
    for (int q = 0; q < RN; ++q) {
      const int gn = n0 + tx + q * (TN / RN);
      if (gn >= N) continue;
      T v = acc[p][q];
      if (S) v *= S[(long long)gm * N + gn];
      C[(long long)gm * ldc + gn] = v;
    }
  }
}

template <typename T>
inline int gemm(T* C, int ldc, const T* A, int lda, const T* B, int ldb, const T* S, int M, int N,
                int K, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0 || M > 65535 * TM || lda < K || ldb < N || ldc < N) {
    axi::set_error("gemm: invalid shape M=%d N=%d K=%d (lda=%d ldb=%d ldc=%d)", M, N, K, lda,
                   ldb, ldc);
    return AXI_ERR_INVALID;
  }
  dim3 grid(axi::ceil_div(N, TN), axi::ceil_div(M, TM));
  gemm_kernel<T><<<grid, THREADS, 0, s>>>(C, ldc, A, lda, B, ldb, S, M, N, K);
  return axi::launch_status("gemm");
}

// out = Er ((Er_inv_w in EzinvT) .* inv_eig) EzT, keeping the reference's
// association A (B C) (kernels/FastDiagonalisationStokesSolver.py:137-156).
template <typename T>
inline int fd_transform_split(T* out, int ld_out, const T* in, int ld_in, const T* Er_inv_w,
                              const T* EzinvT, const T* inv_eig, const T* Er, const T* EzT, T* w1,
                              T* w2, int nr, int nz, cudaStream_t s) {
  AXI_TRY(gemm<T>(w1, nz, in, ld_in, EzinvT, nz, nullptr, nr, nz, nz, s));   // in E_z^-T
  AXI_TRY(gemm<T>(w2, nz, Er_inv_w, nr, w1, nz, inv_eig, nr, nz, nr, s));   // E_r^-1 (.) ./ L
  AXI_TRY(gemm<T>(w1, nz, w2, nz, EzT, nz, nullptr, nr, nz, nz, s));        // (.) E_z^T
  AXI_TRY(gemm<T>(out, ld_out, Er, nr, w1, nz, nullptr, nr, nz, nr, s));    // E_r (.)
  return AXI_OK;
}

template <typename T>
inline int fd_transform(T* out, int ld_out, const T* in, int ld_in, const T* Er_inv_w,
                        const T* EzinvT, const T* inv_eig, const T* Er, const T* EzT, T* work,
                        int nr, int nz, cudaStream_t s) {
  return fd_transform_split<T>(out, ld_out, in, ld_in, Er_inv_w, EzinvT, inv_eig, Er, EzT, work,
                               work + (size_t)nr * nz, nr, nz, s);
}

}  // namespace axi_gemm
