// Orthonormal DCT-II / DCT-III along the rows of (rows, N) double arrays: the
// z-direction products of the double engine's spectral solve when the z
// operator is the Neumann Laplacian (kernels/FastDiagonalisationStokesSolver.py
// :41-97, bc_type homogenous_neumann_along_z_and_r), whose eigenvectors are the
// DCT-II basis vectors c_k cos(pi k (j + 1/2) / N). E_z^-1 x becomes the
// DCT-II of each row and E_z y its DCT-III: O(N log N) per row instead of the
// dense O(N^2) products, with the same psi (it does not depend on which
// eigenbasis diagonalises the operator; the radial products stay dense).
//
// One block transforms a group of rows: Makhoul reordering, a mixed-radix
// (4, 2, 3) Stockham FFT of each row in shared memory, rotation by
// exp(-+ i pi k / 2N). Input and output are row-major, in place of the dense
// products' operands.
#pragma once

#include "axi_common.cuh"

namespace axi_dct64 {

constexpr int MAX_STAGES = 16;
constexpr int ELEMS = 2048;   // complex doubles per buffer; N <= ELEMS
constexpr int THREADS = 256;
// two ping-pong buffers and the twiddle table
constexpr int SMEM_BYTES = 3 * ELEMS * 16;

struct Job {
  int N;                       // row length (nz), even, 2^a 3^b, <= ELEMS
  int rows;                    // rows (nr)
  int nstages;
  int radix[MAX_STAGES];       // Stockham radices, first to last
  const double* in;            // (rows, N) row-major
  double* out;                 // (rows, N) row-major
  const double2* twiddle;      // exp(-2 pi i m / N), m < N
  const double2* rot;          // (cos, sin)(pi k / 2N), k < N
  const double* scale;         // c_k (forward) or 1 / c_k (inverse), k < N
};

// Rows one work item transforms for a row length N.
__host__ __device__ inline int rows_per_item(int N) { return ELEMS / N > 0 ? ELEMS / N : 1; }

// Host: Stockham radices of N (4s, then a 2, then 3s); false if N has another
// factor, is odd or exceeds ELEMS.
bool plan_radices(int N, int* radix, int* nstages);

// Host: launch over `n_items` work items (job, row0, -, -); forward = DCT-II
// (E_z^-1 applied to each row), else DCT-III (E_z).
int launch(const Job* jobs_dev, const int4* items_dev, int n_items, bool forward, cudaStream_t s);

}  // namespace axi_dct64
