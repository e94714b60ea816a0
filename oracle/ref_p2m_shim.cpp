// C entry points over the reference's own particle-to-mesh and mesh-to-particle
// interpolation headers, compiled from its sources in place
// (core/src/particles_to_mesh.hpp, core/src/mesh_to_particles.hpp,
// core/src/interpolation/*_2D.hpp, core/src/particle_kernels/MP4.hpp).
// TEST INFRASTRUCTURE ONLY: used to pin the oracle's restatement. Built into
// oracle/_ref/ by oracle/build.py only where the reference sources are present.
#include <algorithm>  // the header uses std::fill / min / max without including it

#include "mesh_to_particles.hpp"
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

// mesh_to_particles_2D_mp4 (periodic), mesh (n0, n1), particles (p0, p1)
extern "C" void ref_m2p_2d_mp4(const double* in_x, const double* in_y, int n0, int n1,
                               const double* px, const double* py, double* out_x, double* out_y,
                               int p0, int p1, double dx, double dy) {
  mesh_to_particles_2D_mp4<double>(in_x, n0, n1, in_y, n0, n1, px, p0, p1, py, p0, p1, out_x, p0,
                                   p1, out_y, p0, p1, dx, dy);
}

// mesh_to_particles_2D_unbounded_mp4, mesh (n0, n1), particles (p0, p1)
extern "C" void ref_m2p_2d_unbounded_mp4(const double* in_x, const double* in_y, int n0, int n1,
                                         const double* px, const double* py, double* out_x,
                                         double* out_y, int p0, int p1, double dx, double dy) {
  mesh_to_particles_2D_unbounded_mp4<double>(in_x, n0, n1, in_y, n0, n1, px, p0, p1, py, p0, p1,
                                             out_x, p0, p1, out_y, p0, p1, dx, dy);
}
