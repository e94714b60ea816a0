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
  AXI_TRY(axi::check_ptr(what, out, "out"));
  AXI_TRY(axi::check_ptr(what, in, "in"));
  AXI_TRY(axi::check_ptr(what, work, "work"));
  AXI_TRY(axi::check_ptr(what, Er_inv_w, "Er_inv_w"));
  AXI_TRY(axi::check_ptr(what, EzinvT, "EzinvT"));
  AXI_TRY(axi::check_ptr(what, inv_eig, "inv_eig"));
  AXI_TRY(axi::check_ptr(what, Er, "Er"));
  AXI_TRY(axi::check_ptr(what, EzT, "EzT"));
  return axi_gemm::fd_transform<double>(out, ld_out, in, ld_in, Er_inv_w, EzinvT, inv_eig, Er,
                                        EzT, work, nr, nz, axi::as_stream(stream));
}

// ---------------------------------------------------------------------------
// Allocation-free variant of axi_fd_transform_f64.
//
// Some callers cannot call cudaMalloc: a host whose device memory belongs to
// another allocator that has already reserved it, so this library may not ask
// the driver for more.
// For them the two intermediate (nr, nz) products live in this file-scope
// device array instead of caller-provided scratch. It holds
// AXI_FD_STATIC_MAX_CELLS cells per product and stays resident on every GPU
// that loads the library until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

namespace {

constexpr long long kFdStaticCells = 1LL << 19;  // per product: 512 x 1024 cells
static __device__ __align__(256) double g_fd_static_scratch[2 * kFdStaticCells];

// The driver's cuCtxGetCurrent, taken through the runtime (no -lcuda link).
using CtxGetCurrentFn = int (*)(void**);
CtxGetCurrentFn ctx_get_current_fn() {
  static CtxGetCurrentFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(p);
  });
  return fn;
}

// Device address of the array on each device, looked up with that device
// current (the host-side symbol is only a stand-in). It is cached per device
// together with the context it was looked up in: after a device reset the
// primary context is a new one, and the address is looked up again.
double* fd_static_scratch(const char* what) {
  static std::mutex mu;
  static double* addr[128] = {nullptr};
  static void* ctx_of[128] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) {
    axi::set_error("%s: no current CUDA device", what);
    return nullptr;
  }
  const CtxGetCurrentFn get = ctx_get_current_fn();
  auto current = [get]() -> void* {
    void* c = nullptr;
    return (get && get(&c) == 0) ? c : nullptr;
  };
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev] || ctx_of[dev] != current()) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_fd_static_scratch);
    if (e != cudaSuccess || !p) {
      axi::set_error("%s: cudaGetSymbolAddress failed: %s", what, cudaGetErrorString(e));
      return nullptr;
    }
    addr[dev] = static_cast<double*>(p);
    ctx_of[dev] = current();  // the context the lookup made current
  }
  return addr[dev];
}

}  // namespace

extern "C" int64_t axi_fd_transform_static_max_cells(void) { return kFdStaticCells; }

extern "C" int axi_fd_transform_static_f64(double* out, int ld_out, const double* in, int ld_in,
                                           const double* Er_inv_w, const double* EzinvT,
                                           const double* inv_eig, const double* Er,
                                           const double* EzT, int nr, int nz, void* stream) {
  axi::clear_error();
  const char* what = "fd_transform_static";
  AXI_TRY(axi::check_grid(what, nr, nz, 1, 1));
  if ((long long)nr * nz > kFdStaticCells) {
    axi::set_error("%s: grid %d x %d has %lld cells, more than the static scratch holds (%lld)",
                   what, nr, nz, (long long)nr * nz, kFdStaticCells);
    return AXI_ERR_INVALID;
  }
  AXI_TRY(axi::check_ptr(what, out, "out"));
  AXI_TRY(axi::check_ptr(what, in, "in"));
  AXI_TRY(axi::check_ptr(what, Er_inv_w, "Er_inv_w"));
  AXI_TRY(axi::check_ptr(what, EzinvT, "EzinvT"));
  AXI_TRY(axi::check_ptr(what, inv_eig, "inv_eig"));
  AXI_TRY(axi::check_ptr(what, Er, "Er"));
  AXI_TRY(axi::check_ptr(what, EzT, "EzT"));
  double* scratch = fd_static_scratch(what);
  if (!scratch) return AXI_ERR_CUDA;
  // Both products are written in full before they are read, so nothing left
  // by an earlier call needs clearing. The second product starts at a fixed
  // offset so that the layout does not depend on the grid.
  return axi_gemm::fd_transform_split<double>(out, ld_out, in, ld_in, Er_inv_w, EzinvT, inv_eig,
                                              Er, EzT, scratch, scratch + kFdStaticCells, nr, nz,
                                              axi::as_stream(stream));
}
