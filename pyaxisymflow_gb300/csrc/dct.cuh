// Orthonormal DCT-II / DCT-III along the rows of (rows, N) float arrays, the
// z-direction products of the spectral Poisson solve when the z operator is
// the uniform Neumann Laplacian (FD matrix of
// kernels/FastDiagonalisationStokesSolver.py:41-97 with bc_type
// homogenous_neumann_along_z_and_r): its eigenvectors are the DCT-II basis
// vectors c_k cos(pi k (j + 1/2) / N) (c_0 = sqrt(1/N), c_k = sqrt(2/N)), so
// E_z^-1 x (= E_z^T x) is the orthonormal DCT-II of x and E_z y its inverse.
// psi does not depend on which eigenbasis diagonalises the operator, so the
// O(N^2) dense products become O(N log N) transforms.
//
// Each transform reorders the row (Makhoul: even samples forward, odd
// samples backward), runs a complex mixed-radix (4, 2, 3) Stockham FFT in
// shared memory and rotates by exp(-+ i pi k / 2N). Output is written
// transposed, (N, rows), as the TF32 operand pair of the radial tensor-core
// product that follows.
#pragma once

#include <cstdint>

#include "axi_common.cuh"

namespace axi_dct {

constexpr int MAX_STAGES = 16;
constexpr int ELEMS = 4096;                      // complex values per shared buffer
constexpr int THREADS = 256;
// two ping-pong buffers of float2 and the twiddle table (N <= ELEMS)
constexpr int SMEM_BYTES = 3 * ELEMS * 8;

// One row-transform problem (one case).
struct DctJob {
  int N;                       // row length (nz), even, 2^a 3^b, <= ELEMS
  int rows;                    // rows of the input (nr)
  int nstages;
  int radix[MAX_STAGES];       // Stockham radices, first to last
  const float* in;             // (rows, N) row-major
  float* out_hi;               // (N, rows) row-major: TF32 hi part
  float* out_lo;               // (N, rows): TF32 remainder
  const float2* twiddle;       // exp(-2 pi i m / N), m < N
  const float2* rot;           // (cos, sin)(pi k / 2N), k < N
  const float* scale;          // c_k (forward) or 1 / c_k (inverse), k < N
  const float* row_scale;      // inverse: (rows, N) elementwise factor applied to
                               // the input before 1 / c_k (the spectral
                               // inverse), or nullptr
  // Forward with psi (iterative refinement of the Poisson solve): the rows
  // transformed are the residual x = in - (A psi) / r of the discrete
  // operator A = A_r (x) I + I (x) A_z of the solve (Neumann z ends, axis
  // row 0, Neumann outer row), so the solve of x is the correction to add to
  // psi. rinv2dx = 1 / (2 dx r_i), rinv2 = 1 / r_i^2 per row.
  const float* psi;
  const float* psi_lo;         // psi is the pair psi + psi_lo
  const float* rinv2dx;
  const float* rinv2;
  float two_over_dx;           // 2 / dx
  float inv_2dx;               // 1 / (2 dx)
};

// Rows one work item of the generic path transforms for a row length N.
__host__ __device__ inline int rows_per_item(int N) { return ELEMS / N > 0 ? ELEMS / N : 1; }

// Register-resident four-step FFT lengths N = N1 x N2 (one warp per pair
// of real rows): N1 of the first pass, 0 when N has no such path.
__host__ __device__ constexpr int reg_n1(int N) {
  return N == 256 ? 16 : N == 512 ? 16 : N == 768 ? 24 : N == 1024 ? 32 : 0;
}
// Complex values per warp buffer of the register path: at least the
// N + N1 - 1 the four-step exchange addresses, rounded up to 2 (mod 16) so
// that every buffer starts 16-byte aligned and the transposed stores (four
// rows of one column from two buffers per half-warp) touch distinct banks.
__host__ __device__ constexpr int reg_buf(int N) {
  return ((N + reg_n1(N) - 1 - 2 + 15) / 16) * 16 + 2;
}
// Twiddle table of the register path: exp(-2 pi i m / N) at index
// m + m / 16 (one pad entry per 16, so the strided inter-pass reads
// tw[n2 k1] spread over the banks).
__host__ __device__ constexpr int reg_tw_index(int m) { return m + (m >> 4); }
__host__ __device__ constexpr int reg_tw_size(int N) { return N + N / 16; }
// Warps (pairs of real rows) per work item of the register path: the warp
// buffers and the padded twiddle table within 3 x ELEMS complex values.
__host__ __device__ constexpr int reg_warps(int N) {
  return reg_n1(N) == 0 ? 0
                        : ((3 * ELEMS - reg_tw_size(N)) / reg_buf(N) < THREADS / 32
                               ? (3 * ELEMS - reg_tw_size(N)) / reg_buf(N)
                               : THREADS / 32);
}

// Rows per work item for row length N (lengths with a specialised kernel
// pack two real rows per complex transform).
__host__ __device__ inline int rows_for(int N) {
  if (reg_n1(N)) return 2 * reg_warps(N);
  if (N == 1536 || N == 2048) return 2 * (ELEMS / N);
  return rows_per_item(N);
}

// Host: Stockham radices of N (4s, then a 2, then 3s); false if N has
// another factor or needs more than MAX_STAGES stages.
bool plan_radices(int N, int* radix, int* nstages);

// Host: launch over `n_items` work items (job, row0, -, -); forward = DCT-II
// (E_z^T x), else DCT-III (E_z y).
// `prefetch_waves`: L2 prefetch distance in resident waves (0: one, -1: none).
int launch(const DctJob* jobs_dev, const int4* items_dev, int n_items, bool forward,
           cudaStream_t s, int prefetch_waves = 0);

}  // namespace axi_dct
