"""Level-set reinitialisation on the device, for the reference's call site
examples/SoftSphereStreaming/soft_sphere_streaming.py:195-199 (and
examples/SoftSphereInTaylorGreenVortex/soft_sphere_in_taylor_green_vortex.py:160):

    bad_phi[...] = ball_phi
    ball_phi = skfmm.distance(ball_phi, dx=dx, narrow=reinit_band)
    idx = ball_phi.mask
    ball_phi[idx] = bad_phi[idx]

is reinitialise_level_set(ball_phi, dx, reinit_band) (in place). distance()
returns the distance field and the band mask separately. The zero contour is
the marching-squares reconstruction of phi and band points take their exact
distance to it (scikit-fmm marches the eikonal equation instead; both are
second-order accurate for a smooth interface, and scikit-fmm is not
available to compare against bit for bit).
"""
import torch

from .. import _native as N

_work = {}


def _scratch(nr, nz, device):
    key = (nr, nz, device)
    if key not in _work:
        _work[key] = torch.empty(int(N.lib().axi_level_set_work_bytes(nr, nz)),
                                 dtype=torch.uint8, device=device)
    return _work[key]


def distance(phi, dx, narrow, out=None):
    """Signed distance to the zero contour of phi (a (nr, nz) float64 CUDA
    tensor) for points within `narrow` of it, phi's own value elsewhere.
    Returns (out, in_band) with in_band a bool tensor (True inside the band)."""
    if out is None:
        out = torch.empty_like(phi)
    N.require(phi, out, shape=phi.shape, dtype=torch.float64, names=("phi", "out"))
    if phi.dim() != 2:
        raise ValueError("phi must be a 2-D (nr, nz) field")
    if out.data_ptr() == phi.data_ptr():
        raise ValueError("out must not alias phi")
    nr, nz = phi.shape
    band = torch.empty((nr, nz), dtype=torch.uint8, device=phi.device)
    N.call("axi_level_set_distance_f64", N.ptr(out), N.ptr(phi), nr, nz, float(dx),
           float(narrow), N.ptr(band), N.ptr(_scratch(nr, nz, phi.device)), N.stream_of(phi))
    return out, band.bool()


def reinitialise_level_set(phi, dx, narrow):
    """In place: phi becomes the signed distance to its zero contour within
    `narrow`, and keeps its values outside the band."""
    d, _ = distance(phi, dx, narrow)
    phi.copy_(d)
    return phi
