"""Test infrastructure (the oracle): a host restatement of the device
level-set distance (pyaxisymflow_gb300/csrc/levelset.cu), which stands in for
scikit-fmm's skfmm.distance at
examples/SoftSphereStreaming/soft_sphere_streaming.py:197.

scikit-fmm (2022.8.15) is not installed here and no reference test pins its
output, so this restatement is checked against the exact distance of known
interfaces (tests) rather than against scikit-fmm: parity with scikit-fmm is
unpinned. The operations and their order follow the device code exactly
(numpy float64 elementwise arithmetic, no contraction), so the device result
must match this one bit for bit.
"""
import math

import numpy as np


def segments(phi):
    """Marching-squares segments of the zero contour: list of
    (ci, cj, y0, x0, y1, x1) in grid units."""
    phi = np.asarray(phi, dtype=np.float64)
    nr, nz = phi.shape
    out = []
    for i in range(nr - 1):
        for j in range(nz - 1):
            p00, p01 = phi[i, j], phi[i, j + 1]
            p10, p11 = phi[i + 1, j], phi[i + 1, j + 1]
            s00, s01, s10, s11 = p00 < 0, p01 < 0, p10 < 0, p11 < 0
            has = [s00 != s01, s01 != s11, s10 != s11, s00 != s10]
            fi, fj = float(i), float(j)
            pts = [None] * 4
            if has[0]:
                pts[0] = (fi, fj + p00 / (p00 - p01))
            if has[1]:
                pts[1] = (fi + p01 / (p01 - p11), fj + 1.0)
            if has[2]:
                pts[2] = (fi + 1.0, fj + p10 / (p10 - p11))
            if has[3]:
                pts[3] = (fi + p00 / (p00 - p10), fj)
            n = sum(has)
            if n == 2:
                a, b = [k for k in range(4) if has[k]]
                out.append((i, j) + pts[a] + pts[b])
            elif n == 4:
                s = ((p00 + p01) + p10) + p11
                if (s < 0) == s00:
                    out.append((i, j) + pts[0] + pts[1])
                    out.append((i, j) + pts[2] + pts[3])
                else:
                    out.append((i, j) + pts[0] + pts[3])
                    out.append((i, j) + pts[1] + pts[2])
    return out


def _dist2(py, px, y0, x0, y1, x1):
    ey, ex = y1 - y0, x1 - x0
    wy, wx = py - y0, px - x0
    l2 = ey * ey + ex * ex
    with np.errstate(invalid="ignore", divide="ignore"):
        t = (wy * ey + wx * ex) / l2
    t = np.clip(t, 0.0, 1.0)
    qy, qx = y0 + t * ey, x0 + t * ex
    dy, dx = py - qy, px - qx
    d2 = dy * dy + dx * dx
    return np.where(l2 == 0.0, wy * wy + wx * wx, d2)


def distance(phi, dx, narrow):
    """(out, in_band) as the device computes them."""
    phi = np.asarray(phi, dtype=np.float64)
    nr, nz = phi.shape
    segs = np.array(segments(phi), dtype=np.float64).reshape(-1, 6)
    W = int(math.ceil(narrow / dx))
    out = phi.copy()
    band = np.zeros(phi.shape, dtype=bool)
    for i in range(nr):
        for j in range(nz):
            v = phi[i, j]
            if v == 0.0:
                best = 0.0
            else:
                sel = ((segs[:, 0] >= i - W - 1) & (segs[:, 0] <= i + W)
                       & (segs[:, 1] >= j - W - 1) & (segs[:, 1] <= j + W))
                if not sel.any():
                    continue
                s = segs[sel]
                best = float(np.min(_dist2(float(i), float(j), s[:, 2], s[:, 3], s[:, 4], s[:, 5])))
            d = math.sqrt(best) * dx
            if d <= narrow:
                out[i, j] = -d if v < 0 else d
                band[i, j] = True
    return out, band
