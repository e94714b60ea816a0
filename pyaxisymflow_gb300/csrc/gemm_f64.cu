// FP64 GEMM and the fast-diagonalisation spectral transform of the plain path
// (kernels/FastDiagonalisationStokesSolver.py:130-156,
// kernels/FastDiagonalisationPotentialSolver.py:119-145,
// kernels/implicit_diffusion_solver.py:108-143).
#include "gemm_simt.cuh"

extern "C" int axi_dgemm_f64(double* C, int ldc, const double* A, int lda, const double* B,
                             int ldb, const double* S, int M, int N, int K, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("dgemm", C, "C"));
  AXI_TRY(axi::check_ptr("dgemm", A, "A"));
  AXI_TRY(axi::check_ptr("dgemm", B, "B"));
  return axi_gemm::gemm<double>(C, ldc, A, lda, B, ldb, S, M, N, K, axi::as_stream(stream));
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
  return axi_gemm::fd_transform<double>(out, ld_out, in, ld_in, Er_inv_w, EzinvT, inv_eig, Er,
                                        EzT, work, nr, nz, axi::as_stream(stream));
}
