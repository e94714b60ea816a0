// C entry points over the reference's own least-squares extrapolation header,
// compiled from its sources in place (core/src/extrapolate_using_least_squares.hpp,
// core/src/lstsq/least_squares.hpp). TEST INFRASTRUCTURE ONLY: used to pin the
// oracle's restatement. Built into oracle/_ref/ by oracle/build.py only where
// the reference sources are present.
#include "extrapolate_using_least_squares.hpp"

extern "C" void ref_extrapolate_till_first_order(short* current_flag, const short* target_flag,
                                                  double* eta_x, double* eta_y,
                                                  const double* grid_x, const double* grid_y,
                                                  int n0, int n1, int nx, int ny) {
  extrapolate_using_least_squares_till_first_order<short, double>(
      current_flag, n0, n1, target_flag, n0, n1, eta_x, n0, n1, eta_y, n0, n1,
      grid_x, nx, grid_y, ny);
}

// Runs lstsq::gauss_elimination<3, 2, 9> on a caller-provided 3x5 augmented
// matrix (row-major) and writes the 2x3 solution.
extern "C" void ref_gauss_elimination_3x2(const double* aug, double* sol) {
  double A[3][5];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 5; ++j) A[i][j] = aug[i * 5 + j];
  double out[2][9];
  lstsq::gauss_elimination<3, 2, 9>(A, out);
  for (int c = 0; c < 2; ++c)
    for (int i = 0; i < 3; ++i) sol[c * 3 + i] = out[c][i];
}
