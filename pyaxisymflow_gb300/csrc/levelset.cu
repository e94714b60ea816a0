// Level-set reinitialisation on the device: the signed distance to the zero
// contour of phi within a narrow band, the role of scikit-fmm's
// skfmm.distance(phi, dx=dx, narrow=band) at the reference's call site
// (examples/SoftSphereStreaming/soft_sphere_streaming.py:195-199, where the
// points outside the band keep their previous values).
//
// scikit-fmm marches the eikonal equation outward from the interface on the
// host. Here the interface is reconstructed once as marching-squares segments
// (zero crossings linearly interpolated along the cell edges; a saddle cell
// joins its crossings by the sign of the cell's corner sum), and every point
// then takes its exact Euclidean distance to the nearest segment within the
// band: independent per point, O(dx^2) accurate for a smooth interface.
// All arithmetic is FP64 without contraction, in grid units (the distance is
// scaled by dx at the end), so a host restatement reproduces it bit for bit.
#include "axi_common.cuh"

namespace {

// one interface segment, (y0, x0) - (y1, x1) in grid units
struct Seg {
  double y0, x0, y1, x1;
};

struct LsLayout {
  size_t cnt, seg, total;
};

size_t ls_align(size_t x) { return (x + 255) / 256 * 256; }

LsLayout ls_layout(int nr, int nz) {
  const size_t cells = (size_t)(nr - 1) * (nz - 1);
  LsLayout L;
  L.cnt = 0;
  L.seg = ls_align(cells * sizeof(int));
  L.total = L.seg + ls_align(cells * 2 * sizeof(Seg));
  return L;
}

// zero crossing on the edge from value va to value vb: the fraction along it
__device__ __forceinline__ double crossing(double va, double vb) {
  return __ddiv_rn(va, __dsub_rn(va, vb));
}

// Segments of cell (i, j) (corners (i, j), (i, j+1), (i+1, j+1), (i+1, j));
// a segment is (y0, x0, y1, x1) in grid units. Negative values are inside
// one region, values >= 0 in the other.
__global__ void ls_segments_kernel(const double* __restrict__ phi, int nr, int nz,
                                   int* __restrict__ cnt, Seg* __restrict__ seg) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= nz - 1 || i >= nr - 1) return;
  const double p00 = phi[(long long)i * nz + j], p01 = phi[(long long)i * nz + j + 1];
  const double p10 = phi[(long long)(i + 1) * nz + j], p11 = phi[(long long)(i + 1) * nz + j + 1];
  const bool s00 = p00 < 0, s01 = p01 < 0, s10 = p10 < 0, s11 = p11 < 0;
  const double fi = (double)i, fj = (double)j;
  // crossings in edge order bottom, right, top, left
  double cy[4], cx[4];
  bool has[4] = {s00 != s01, s01 != s11, s10 != s11, s00 != s10};
  if (has[0]) { cy[0] = fi; cx[0] = __dadd_rn(fj, crossing(p00, p01)); }
  if (has[1]) { cy[1] = __dadd_rn(fi, crossing(p01, p11)); cx[1] = fj + 1.0; }
  if (has[2]) { cy[2] = fi + 1.0; cx[2] = __dadd_rn(fj, crossing(p10, p11)); }
  if (has[3]) { cy[3] = __dadd_rn(fi, crossing(p00, p10)); cx[3] = fj; }
  const int n = (int)has[0] + (int)has[1] + (int)has[2] + (int)has[3];
  const long long c = (long long)i * (nz - 1) + j;
  if (n == 2) {
    int a = 0;
    while (!has[a]) ++a;
    int b = a + 1;
    while (!has[b]) ++b;
    seg[2 * c] = Seg{cy[a], cx[a], cy[b], cx[b]};
  } else if (n == 4) {
    const double sum = __dadd_rn(__dadd_rn(__dadd_rn(p00, p01), p10), p11);
    if ((sum < 0) == s00) {
      // the corner-(0,0) sign joins (0,0) and (1,1): cut off corners (0,1) and (1,0)
      seg[2 * c] = Seg{cy[0], cx[0], cy[1], cx[1]};
      seg[2 * c + 1] = Seg{cy[2], cx[2], cy[3], cx[3]};
    } else {
      seg[2 * c] = Seg{cy[0], cx[0], cy[3], cx[3]};
      seg[2 * c + 1] = Seg{cy[1], cx[1], cy[2], cx[2]};
    }
  }
  cnt[c] = n / 2;
}

// squared distance (grid units) from (py, px) to segment s
__device__ __forceinline__ double seg_dist2(double py, double px, const Seg& s) {
  const double ey = __dsub_rn(s.y1, s.y0), ex = __dsub_rn(s.x1, s.x0);
  const double wy = __dsub_rn(py, s.y0), wx = __dsub_rn(px, s.x0);
  const double l2 = __dadd_rn(__dmul_rn(ey, ey), __dmul_rn(ex, ex));
  if (l2 == 0.0) return __dadd_rn(__dmul_rn(wy, wy), __dmul_rn(wx, wx));
  double t = __ddiv_rn(__dadd_rn(__dmul_rn(wy, ey), __dmul_rn(wx, ex)), l2);
  t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
  const double qy = __dadd_rn(s.y0, __dmul_rn(t, ey)), qx = __dadd_rn(s.x0, __dmul_rn(t, ex));
  const double dy = __dsub_rn(py, qy), dx = __dsub_rn(px, qx);
  return __dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dx, dx));
}

__global__ void ls_distance_kernel(const double* __restrict__ phi, int nr, int nz, double dx,
                                   double narrow, int W, const int* __restrict__ cnt,
                                   const Seg* __restrict__ seg, double* __restrict__ out,
                                   unsigned char* __restrict__ in_band) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= nz || i >= nr) return;
  const long long p = (long long)i * nz + j;
  const double v = phi[p];
  double best = -1.0;
  if (v == 0.0) {
    best = 0.0;
  } else {
    const int c0 = max(i - W - 1, 0), c1 = min(i + W, nr - 2);
    const int d0 = max(j - W - 1, 0), d1 = min(j + W, nz - 2);
    const double py = (double)i, px = (double)j;
    for (int ci = c0; ci <= c1; ++ci) {
      for (int cj = d0; cj <= d1; ++cj) {
        const long long c = (long long)ci * (nz - 1) + cj;
        const int n = cnt[c];
        for (int q = 0; q < n; ++q) {
          const double d2 = seg_dist2(py, px, seg[2 * c + q]);
          if (best < 0.0 || d2 < best) best = d2;
        }
      }
    }
  }
  double d = -1.0;
  if (best >= 0.0) d = __dmul_rn(__dsqrt_rn(best), dx);
  if (d >= 0.0 && d <= narrow) {
    out[p] = v < 0 ? -d : d;
    if (in_band) in_band[p] = 1;
  } else {
    out[p] = v;
    if (in_band) in_band[p] = 0;
  }
}

}  // namespace

extern "C" int64_t axi_level_set_work_bytes(int nr, int nz) {
  if (nr < 2 || nz < 2) return 0;
  return (int64_t)ls_layout(nr, nz).total;
}

extern "C" int axi_level_set_distance_f64(double* out, const double* phi, int nr, int nz,
                                          double dx, double narrow, unsigned char* in_band,
                                          void* work, void* stream) {
  axi::clear_error();
  AXI_TRY(axi::check_ptr("level_set_distance", out, "out"));
  AXI_TRY(axi::check_ptr("level_set_distance", phi, "phi"));
  AXI_TRY(axi::check_ptr("level_set_distance", work, "work"));
  AXI_TRY(axi::check_grid("level_set_distance", nr, nz, 2, 2));
  if (!(dx > 0.0) || !(narrow >= 0.0) || nr > 65535 || narrow / dx > 4096.0) {
    axi::set_error("level_set_distance: dx %g, narrow %g or grid %d x %d invalid (band at most "
                   "4096 cells)", dx, narrow, nr, nz);
    return AXI_ERR_INVALID;
  }
  if (out == phi) {
    axi::set_error("level_set_distance: out must not alias phi");
    return AXI_ERR_INVALID;
  }
  const LsLayout L = ls_layout(nr, nz);
  char* wb = static_cast<char*>(work);
  int* cnt = reinterpret_cast<int*>(wb + L.cnt);
  Seg* seg = reinterpret_cast<Seg*>(wb + L.seg);
  cudaStream_t s = axi::as_stream(stream);
  const int W = (int)ceil(narrow / dx);
  ls_segments_kernel<<<dim3((nz - 1 + 127) / 128, nr - 1), 128, 0, s>>>(phi, nr, nz, cnt, seg);
  ls_distance_kernel<<<dim3((nz + 127) / 128, nr), 128, 0, s>>>(phi, nr, nz, dx, narrow, W, cnt,
                                                               seg, out, in_band);
  return axi::launch_status("level_set_distance");
}
