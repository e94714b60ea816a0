// C entry points over the reference's own particle-to-mesh interpolation
// header, compiled from its sources in place (core/src/particles_to_mesh.hpp,
// core/src/interpolation/particles_to_mesh_2D.hpp, core/src/particle_kernels/MP4.hpp).
// TEST INFRASTRUCTURE ONLY: used to pin the oracle's restatement. Built into
// oracle/_ref/ by oracle/build.py only where the reference sources are present.
#include <algorithm>  // the header uses std::fill / min / max without including it

#include "particles_to_mesh.hpp"

// particles_to_mesh_2D_mp4 (periodic in both directions), arrays (n0, n1)
extern "C" void ref_p2m_2d_mp4(const double* px, const double* py, const double* vin,
                               double* out, int n0, int n1, double dx, double dy) {
  particles_to_mesh_2D_mp4<double>(px, n0, n1, py, n0, n1, vin, n0, n1, out, n0, n1, dx, dy);
}

// particles_to_mesh_2D_unbounded_mp4, arrays (n0, n1)
extern "C" void ref_p2m_2d_unbounded_mp4(const double* px, const double* py, const double* vin,
                                         double* out, int n0, int n1, double dx, double dy) {
  particles_to_mesh_2D_unbounded_mp4<double>(px, n0, n1, py, n0, n1, vin, n0, n1, out, n0, n1,
                                             dx, dy);
}
