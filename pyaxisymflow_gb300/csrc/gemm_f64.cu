// FP64 GEMM and the fast-diagonalisation spectral transform of the plain path.
//
// GB300 executes FP64 at about 1 TFLOP/s (DFMA and DMMA alike), 1/70 of its
// FP32 rate, so the four dense transforms of a spectral solve are bound by the
// FP64 pipe, not by memory. The kernel below is a register-tiled SIMT DFMA
// GEMM: each thread keeps a 4x4 accumulator tile, operands are staged through
// shared memory in K-slices, and the tile size is picked so that the grid
// covers the 152 SMs even for the smallest solves (256 x 512 fields).
//
// kernels/FastDiagonalisationStokesSolver.py:137-156 evaluates
//   buf = E_r^-1 (r .* w E_z^-T);  buf .*= 1/Lambda;  psi = E_r (buf E_z^T)
// (numpy multi_dot picks A (B C) for these equally costed triples); the
// transform below keeps that association, with diag(r) folded into E_r^-1 by
// the caller.
#include "axi_common.cuh"

namespace {

constexpr int TM = 32;   // rows of C per block
constexpr int TN = 32;   // cols of C per block
constexpr int TK = 32;   // K slice staged in shared memory
constexpr int RM = 4;    // rows per thread
constexpr int RN = 4;    // cols per thread
constexpr int THREADS = (TM / RM) * (TN / RN);  // 64

// C[M,N] = A[M,K] B[K,N] (row-major with row strides ldc/lda/ldb), optionally
// .* S[M,N] (row stride N).
__global__ void __launch_bounds__(THREADS) dgemm_kernel(double* __restrict__ C, int ldc,
                                                        const double* __restrict__ A, int lda,
                                                        const double* __restrict__ B, int ldb,
                                                        const double* __restrict__ S, int M,
                                                        int N, int K) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN];
  const int tx = threadIdx.x % (TN / RN);
  const int ty = threadIdx.x / (TN / RN);
  const int m0 = blockIdx.y * TM;
  const int n0 = blockIdx.x * TN;
  double acc[RM][RN];
#pragma unroll
  for (int a = 0; a < RM; ++a)
#pragma unroll
    for (int b = 0; b < RN; ++b) acc[a][b] = 0.0;

  for (int k0 = 0; k0 < K; k0 += TK) {
    // A tile: TM x TK, stored transposed so the inner loop reads a column.
    for (int e = threadIdx.x; e < TM * TK; e += THREADS) {
      const int r = e / TK, kk = e % TK;
      const int gm = m0 + r, gk = k0 + kk;
      As[kk][r] = (gm < M && gk < K) ? A[(long long)gm * lda + gk] : 0.0;
    }
    for (int e = threadIdx.x; e < TK * TN; e += THREADS) {
      const int kk = e / TN, cidx = e % TN;
      const int gk = k0 + kk, gn = n0 + cidx;
      Bs[kk][cidx] = (gk < K && gn < N) ? B[(long long)gk * ldb + gn] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < TK; ++kk) {
      double a[RM], b[RN];
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
      double v = acc[p][q];
      if (S) v *= S[(long long)gm * N + gn];
      C[(long long)gm * ldc + gn] = v;
    }
  }
}

int dgemm(double* C, int ldc, const double* A, int lda, const double* B, int ldb,
          const double* S, int M, int N, int K, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0 || M > 65535 * TM || lda < K || ldb < N || ldc < N) {
    axi::set_error("dgemm: invalid shape M=%d N=%d K=%d (lda=%d ldb=%d ldc=%d)", M, N, K, lda,
                   ldb, ldc);
    return AXI_ERR_INVALID;
  }
  dim3 grid(axi::ceil_div(N, TN), axi::ceil_div(M, TM));
  dgemm_kernel<<<grid, THREADS, 0, s>>>(C, ldc, A, lda, B, ldb, S, M, N, K);
  return axi::launch_status("dgemm");
}

}  // namespace

extern "C" int axi_dgemm_f64(double* C, int ldc, const double* A, int lda, const double* B,
                             int ldb, const double* S, int M, int N, int K, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("dgemm", C, "C"));
  AXI_TRY(axi::check_ptr("dgemm", A, "A"));
  AXI_TRY(axi::check_ptr("dgemm", B, "B"));
  return dgemm(C, ldc, A, lda, B, ldb, S, M, N, K, axi::as_stream(stream));
}

extern "C" int axi_fd_transform_f64(double* out, int ld_out, const double* in, int ld_in,
                                    const double* Er_inv_w, const double* EzinvT,
                                    const double* inv_eig, const double* Er, const double* EzT,
                                    double* work, int nr, int nz, void* stream) {
  axi::clear_error();
  const char* what = "fd_transform";
  AXI_TRY(axi::check_grid(what, nr, nz, 1, 1));
  AXI_TRY(axi::check_ptr(what, work, "work"));
  AXI_TRY(axi::check_ptr(what, Er_inv_w, "Er_inv_w"));
  AXI_TRY(axi::check_ptr(what, EzinvT, "EzinvT"));
  AXI_TRY(axi::check_ptr(what, inv_eig, "inv_eig"));
  AXI_TRY(axi::check_ptr(what, Er, "Er"));
  AXI_TRY(axi::check_ptr(what, EzT, "EzT"));
  cudaStream_t s = axi::as_stream(stream);
  double* w1 = work;
  double* w2 = work + (size_t)nr * nz;
  AXI_TRY(dgemm(w1, nz, in, ld_in, EzinvT, nz, nullptr, nr, nz, nz, s));     // in E_z^-T
  AXI_TRY(dgemm(w2, nz, Er_inv_w, nr, w1, nz, inv_eig, nr, nz, nr, s));     // E_r^-1 (.) ./ Lambda
  AXI_TRY(dgemm(w1, nz, w2, nz, EzT, nz, nullptr, nr, nz, nz, s));          // (.) E_z^T
  AXI_TRY(dgemm(out, ld_out, Er, nr, w1, nz, nullptr, nr, nz, nr, s));      // E_r (.)
  return AXI_OK;
}
