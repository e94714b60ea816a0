// Particle-to-mesh interpolation with the MP4 kernel (the remeshing step of
// the remeshed vortex method, kernels/advect_particle.py), deterministic and
// bit-identical to the sequential reference
// (core/src/interpolation/particles_to_mesh_2D.hpp:14-324).
//
// The reference scatters every particle's 4 x 4 stencil into the mesh in
// particle order. Here every mesh point gathers instead: it visits the
// particles that can reach it in increasing particle index and adds their
// contributions with unfused double operations, so each mesh value is the
// same sum in the same order. Which particles can reach a mesh point follows
// from the particle array being indexed like the mesh (particle (j, i) starts
// at mesh point (j, i), as in the reference's remeshing, which resets the
// particles to the mesh every step): a particle that moved less than one
// cell along each axis anchors its stencil at its own index or the next one,
// so mesh point (j, i) gathers from particles (j-2..j+2, i-2..i+2). The
// stencil kernel flags any particle that moved further; the result is then
// invalid and the caller is told (axi_p2m_status).
#include "axi_common.cuh"

namespace {

// the four MP4 weights of one particle along one axis
struct alignas(16) Weights4 {
  double v[4];
};

struct P2MLayout {
  size_t h, wx, wy, flag, total;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

P2MLayout p2m_layout(int n0, int n1) {
  const size_t n = (size_t)n0 * n1;
  P2MLayout L;
  size_t o = 0;
  L.h = o;
  o = align_up(o + n * sizeof(int2), 256);
  L.wx = o;
  o = align_up(o + n * sizeof(Weights4), 256);
  L.wy = o;
  o = align_up(o + n * sizeof(Weights4), 256);
  L.flag = o;
  o = align_up(o + 16, 256);
  L.total = o;
  return L;
}

// MP4 (core/src/particle_kernels/MP4.hpp): |x| <= 1 and 1 < |x| <= 2 branches,
// evaluated in the reference's operation order without contraction.
__device__ __forceinline__ double mp4_inner(double t) {
  return __dadd_rn(1.0, __dmul_rn(__dmul_rn(t, t), __dadd_rn(-2.5, __dmul_rn(1.5, t))));
}
__device__ __forceinline__ double mp4_outer(double t) {
  return __dadd_rn(2.0,
                   __dmul_rn(t, __dadd_rn(-4.0, __dmul_rn(t, __dsub_rn(2.5, __dmul_rn(0.5, t))))));
}

// Anchor h (mesh index nearest above the particle on the cell-centred mesh)
// and the four stencil weights along one axis
// (particles_to_mesh_2D.hpp:60-118; slot k has offset k - 2, the outer slots
// 0 and 3 use the outer branch, core/src/particle_kernels/KernelWrapper.hpp:31-47).
__device__ __forceinline__ int mp4_stencil(double pos, double w[4]) {
  const double fl = floor(pos);
  const int h = (pos >= __dadd_rn(fl, 0.5) ? 1 : 0) + (int)fl;
  const double base = __dadd_rn((double)h, 0.5);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double d = fabs(__dsub_rn(pos, __dadd_rn(base, (double)(k - 2))));
    w[k] = (k == 0 || k == 3) ? mp4_outer(d) : mp4_inner(d);
  }
  return h;
}

__global__ void p2m_stencil_kernel(const double* __restrict__ px, const double* __restrict__ py,
                                   int n0, int n1, double dx, double dy, int2* __restrict__ H,
                                   Weights4* __restrict__ WX, Weights4* __restrict__ WY,
                                   int* __restrict__ flag) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (long long)n0 * n1) return;
  const int j = (int)(p / n1), i = (int)(p % n1);
  double wx[4], wy[4];
  const int hx = mp4_stencil(__ddiv_rn(px[p], dx), wx);
  const int hy = mp4_stencil(__ddiv_rn(py[p], dy), wy);
  H[p] = make_int2(hx, hy);
  WX[p] = Weights4{{wx[0], wx[1], wx[2], wx[3]}};
  WY[p] = Weights4{{wy[0], wy[1], wy[2], wy[3]}};
  if (hx - i < 0 || hx - i > 1 || hy - j < 0 || hy - j > 1) atomicOr(flag, 1);
}

// The up to five particle indices m - 2 .. m + 2 along one axis (wrapped when
// periodic, clipped otherwise), in increasing order.
__device__ __forceinline__ int candidates(int m, int n, bool periodic, int out[5]) {
  int c = 0;
  for (int d = -2; d <= 2; ++d) {
    int q = m + d;
    if (periodic) {
      q = (q + n) % n;
    } else if (q < 0 || q >= n) {
      continue;
    }
    int k = c++;
    while (k > 0 && out[k - 1] > q) {  // insertion into the sorted prefix
      out[k] = out[k - 1];
      --k;
    }
    out[k] = q;
  }
  return c;
}

__global__ void p2m_gather_kernel(const double* __restrict__ vin, const int2* __restrict__ H,
                                  const Weights4* __restrict__ WX, const Weights4* __restrict__ WY,
                                  double* __restrict__ out, int n0, int n1, int periodic) {
  const int mi = blockIdx.x * blockDim.x + threadIdx.x;
  const int mj = blockIdx.y;
  if (mi >= n1 || mj >= n0) return;
  int rows[5], cols[5];
  const int nr = candidates(mj, n0, periodic != 0, rows);
  const int nc = candidates(mi, n1, periodic != 0, cols);
  double acc = 0.0;
  for (int a = 0; a < nr; ++a) {
    const int pj = rows[a];
    for (int b = 0; b < nc; ++b) {
      const long long p = (long long)pj * n1 + cols[b];
      const int2 h = H[p];
      int sx = mi - h.x, sy = mj - h.y;
      if (periodic) {
        // the mesh index the reference writes is (h + s + n) % n
        if (sx > n1 / 2) sx -= n1;
        if (sx < -n1 / 2) sx += n1;
        if (sy > n0 / 2) sy -= n0;
        if (sy < -n0 / 2) sy += n0;
      }
      if (sx < -2 || sx > 1 || sy < -2 || sy > 1) continue;
      const double w = __dmul_rn(WY[p].v[sy + 2], WX[p].v[sx + 2]);
      acc = __dadd_rn(acc, __dmul_rn(w, vin[p]));
    }
  }
  out[(long long)mj * n1 + mi] = acc;
}

// Mesh-to-particle MP4 interpolation of two fields
// (core/src/interpolation/mesh_to_particles_2D.hpp:11-183 periodic, :185-420
// unbounded): one thread per particle, the reference's sums in its order
// (each stencil row summed along x from 0.0, then the rows weighted along y
// from 0.0), unfused double operations. The unbounded form clips the stencil
// at the mesh edges but still accumulates all four rows (the clipped rows
// add a zero), as the reference does. Periodic indices wrap like the
// reference's (h + s + n) % n, also for particles more than a period away
// (where the reference's index would be negative).
__device__ __forceinline__ int wrap_index(int a, int n) {
  a %= n;
  return a < 0 ? a + n : a;
}

__global__ void m2p_mp4_kernel(const double* __restrict__ in_x, const double* __restrict__ in_y,
                               int n0, int n1, const double* __restrict__ px,
                               const double* __restrict__ py, double* __restrict__ out_x,
                               double* __restrict__ out_y, long long n_particles, double dx,
                               double dy, int periodic) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_particles) return;
  double wx[4], wy[4];
  const int hx = mp4_stencil(__ddiv_rn(px[p], dx), wx);
  const int hy = mp4_stencil(__ddiv_rn(py[p], dy), wy);
  int sx0 = -2, sx1 = 2, sy0 = -2, sy1 = 2;
  if (!periodic && (hx - 2 < 0 || hy - 2 < 0 || hx + 2 > n1 || hy + 2 > n0)) {
    sx0 = max(-2, -hx);
    sy0 = max(-2, -hy);
    sx1 = min(2, n1 - hx);
    sy1 = min(2, n0 - hy);
  }
  double ps_x[4] = {0.0, 0.0, 0.0, 0.0}, ps_y[4] = {0.0, 0.0, 0.0, 0.0};
  for (int sy = sy0; sy < sy1; ++sy) {
    const long long row = (long long)n1 * (periodic ? wrap_index(hy + sy + n0, n0) : hy + sy);
    double a = 0.0, b = 0.0;
    for (int sx = sx0; sx < sx1; ++sx) {
      const long long m = row + (periodic ? wrap_index(hx + sx + n1, n1) : hx + sx);
      const double w = wx[sx + 2];
      a = __dadd_rn(a, __dmul_rn(w, in_x[m]));
      b = __dadd_rn(b, __dmul_rn(w, in_y[m]));
    }
    ps_x[sy + 2] = a;
    ps_y[sy + 2] = b;
  }
  double acc_x = 0.0, acc_y = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    acc_x = __dadd_rn(acc_x, __dmul_rn(wy[k], ps_x[k]));
    acc_y = __dadd_rn(acc_y, __dmul_rn(wy[k], ps_y[k]));
  }
  out_x[p] = acc_x;
  out_y[p] = acc_y;
}

// kernels/advect_particle.py:20-28 (and :53-61): particles on the mirrored
// (2 nr, nz) domain move with the velocity (mirror rows: u_z even, u_r odd),
// and carry the vorticity (mirror rows odd).
__global__ void particles_prepare_kernel(double* __restrict__ zp, double* __restrict__ rp,
                                         double* __restrict__ vp,
                                         const double* __restrict__ w,
                                         const double* __restrict__ uz,
                                         const double* __restrict__ ur, int nr, int nz,
                                         double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;  // row of the mirrored domain, 0 .. 2 nr - 1
  if (i >= nz || j >= 2 * nr) return;
  const long long d = (long long)j * nz + i;
  if (j >= nr) {
    const long long c = (long long)(j - nr) * nz + i;
    zp[d] = __dadd_rn(zp[d], __dmul_rn(uz[c], dt));
    rp[d] = __dadd_rn(rp[d], __dmul_rn(ur[c], dt));
    vp[d] = w[c];
  } else {
    const long long c = (long long)(nr - 1 - j) * nz + i;
    zp[d] = __dadd_rn(zp[d], __dmul_rn(uz[c], dt));
    rp[d] = __dadd_rn(rp[d], __dmul_rn(-ur[c], dt));
    vp[d] = -w[c];
  }
}

}  // namespace

extern "C" int64_t axi_p2m_mp4_work_bytes(int n0, int n1) {
  if (n0 <= 0 || n1 <= 0) return 0;
  return (int64_t)p2m_layout(n0, n1).total;
}

extern "C" int axi_particles_to_mesh_2d_mp4_f64(const double* px, const double* py,
                                                const double* vin, double* out, int n0, int n1,
                                                double dx, double dy, int periodic, void* work,
                                                void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("particles_to_mesh", px, "particle_positions_x"));
  AXI_TRY(axi::check_ptr("particles_to_mesh", py, "particle_positions_y"));
  AXI_TRY(axi::check_ptr("particles_to_mesh", vin, "input_field_at_particle_positions"));
  AXI_TRY(axi::check_ptr("particles_to_mesh", out, "output_field_at_mesh"));
  AXI_TRY(axi::check_ptr("particles_to_mesh", work, "work"));
  if (n0 < 5 || n1 < 5 || n0 > 65535 || !(dx > 0.0) || !(dy > 0.0)) {
    axi::set_error("particles_to_mesh: grid %d x %d (each side 5 .. 65535) or spacing invalid",
                   n0, n1);
    return AXI_ERR_INVALID;
  }
  const P2MLayout L = p2m_layout(n0, n1);
  char* wb = static_cast<char*>(work);
  int2* H = reinterpret_cast<int2*>(wb + L.h);
  Weights4* WX = reinterpret_cast<Weights4*>(wb + L.wx);
  Weights4* WY = reinterpret_cast<Weights4*>(wb + L.wy);
  int* flag = reinterpret_cast<int*>(wb + L.flag);
  cudaStream_t s = axi::as_stream(stream);
  if (cudaMemsetAsync(flag, 0, sizeof(int), s) != cudaSuccess)
    return axi::launch_status("particles_to_mesh");
  const long long n = (long long)n0 * n1;
  p2m_stencil_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(px, py, n0, n1, dx, dy, H, WX,
                                                                  WY, flag);
  p2m_gather_kernel<<<dim3((n1 + 127) / 128, n0), 128, 0, s>>>(vin, H, WX, WY, out, n0, n1,
                                                                periodic);
  return axi::launch_status("particles_to_mesh");
}

extern "C" int axi_p2m_status(const void* work, int n0, int n1, int* displaced, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("p2m_status", work, "work"));
  AXI_TRY(axi::check_ptr("p2m_status", displaced, "displaced"));
  const P2MLayout L = p2m_layout(n0, n1);
  cudaStream_t s = axi::as_stream(stream);
  if (cudaMemcpyAsync(displaced, static_cast<const char*>(work) + L.flag, sizeof(int),
                      cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return axi::launch_status("p2m_status");
  return AXI_OK;
}

extern "C" int axi_advect_particles_prepare_f64(double* z_particles, double* r_particles,
                                                double* vort_particles, const double* vorticity,
                                                const double* u_z, const double* u_r, int nr,
                                                int nz, double dt, void* stream) {
  axi::clear_error();
  const void* ptrs[] = {z_particles, r_particles, vort_particles, vorticity, u_z, u_r};
  for (const void* p : ptrs) AXI_TRY(axi::check_ptr("advect_particles", p, "field"));
  if (nr <= 0 || nz <= 0 || 2 * nr > 65535) {
    axi::set_error("advect_particles: invalid grid %d x %d", nr, nz);
    return AXI_ERR_INVALID;
  }
  particles_prepare_kernel<<<dim3((nz + 127) / 128, 2 * nr), 128, 0, axi::as_stream(stream)>>>(
      z_particles, r_particles, vort_particles, vorticity, u_z, u_r, nr, nz, dt);
  return axi::launch_status("advect_particles");
}

extern "C" int axi_mesh_to_particles_2d_mp4_f64(const double* input_field_x,
                                                const double* input_field_y, int n0, int n1,
                                                const double* particle_positions_x,
                                                const double* particle_positions_y,
                                                double* output_field_x, double* output_field_y,
                                                int p0, int p1, double dx, double dy,
                                                int periodic, void* stream) {
  axi::clear_error();
  const void* ptrs[] = {input_field_x, input_field_y, particle_positions_x, particle_positions_y,
                        output_field_x, output_field_y};
  for (const void* p : ptrs) AXI_TRY(axi::check_ptr("mesh_to_particles", p, "field"));
  if (n0 <= 0 || n1 <= 0 || p0 <= 0 || p1 <= 0 || !(dx > 0.0) || !(dy > 0.0) ||
      (long long)n0 * n1 >= (1LL << 31)) {
    axi::set_error("mesh_to_particles: mesh %d x %d, particles %d x %d or spacing invalid", n0,
                   n1, p0, p1);
    return AXI_ERR_INVALID;
  }
  const long long n = (long long)p0 * p1;
  m2p_mp4_kernel<<<(unsigned)((n + 255) / 256), 256, 0, axi::as_stream(stream)>>>(
      input_field_x, input_field_y, n0, n1, particle_positions_x, particle_positions_y,
      output_field_x, output_field_y, n, dx, dy, periodic);
  return axi::launch_status("mesh_to_particles");
}
