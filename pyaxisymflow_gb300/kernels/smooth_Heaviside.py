"""Drop-in for pyaxisymflow/kernels/smooth_Heaviside.py:5-14."""
from .. import _native as N


def smooth_Heaviside(H, phi, blend_w):
    """computes a smooth Heaviside function of the level set phi into H."""
    s = N.require(H, phi, shape=H.shape, names=("H", "phi"))
    N.call(f"axi_smooth_heaviside_{s}", N.ptr(H), N.ptr(phi), N.real(s, blend_w), H.numel(),
           N.stream_of(H))
