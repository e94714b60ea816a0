"""Device level-set reinitialisation (the role of skfmm.distance at
examples/SoftSphereStreaming/soft_sphere_streaming.py:197) against the
oracle's restatement, bit for bit, and against exact distances."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _fields():
    n, dx = 64, 1.0 / 64
    y, x = np.meshgrid(np.arange(n) * dx, np.arange(n) * dx, indexing="ij")
    circle = 0.27 - np.sqrt((x - 0.51) ** 2 + (y - 0.47) ** 2)
    yield "distorted circle", circle * (1.5 + 0.4 * np.sin(7 * x) * np.cos(5 * y)), dx
    # two circles almost touching: saddle cells between them
    a = 0.2 - np.sqrt((x - 0.3) ** 2 + (y - 0.5) ** 2)
    b = 0.2 - np.sqrt((x - 0.71) ** 2 + (y - 0.5) ** 2)
    yield "two circles", np.maximum(a, b), dx
    rng = np.random.default_rng(9)
    f = np.zeros_like(x)
    for _ in range(12):
        c, s = rng.uniform(0, 1, 2), rng.uniform(0.05, 0.15)
        f += rng.normal() * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2) / (2 * s * s))
    yield "random field", f - 0.1, dx


@pytest.mark.parametrize("case", [0, 1, 2])
def test_level_set_distance_matches_oracle(case):
    from oracle import levelset
    from pyaxisymflow_gb300.kernels.level_set import distance
    name, phi, dx = list(_fields())[case]
    narrow = 6 * dx
    d_ref, band_ref = levelset.distance(phi, dx, narrow)
    d, band = distance(torch.tensor(phi, device="cuda"), dx, narrow)
    assert np.array_equal(band.cpu().numpy(), band_ref), name
    assert np.array_equal(d.cpu().numpy(), d_ref), name


def test_level_set_distance_is_exact_for_a_sphere():
    """The soft-sphere example's level set, distorted: the reinitialised
    field is the exact distance to the sphere's section within the band."""
    from pyaxisymflow_gb300.kernels.level_set import distance
    nz, nr = 512, 256
    dx = 1.0 / nr
    z = np.linspace(dx / 2, nz * dx - dx / 2, nz)
    r = np.linspace(dx / 2, nr * dx - dx / 2, nr)
    Z, R = np.meshgrid(z, r)
    exact = 0.1 - np.sqrt((Z - 1.0) ** 2 + (R - 0.2) ** 2)
    phi = exact * (1.0 + 0.5 * np.tanh(4 * (Z - 1.0)))
    narrow = 8 * dx
    d, band = distance(torch.tensor(phi, device="cuda"), dx, narrow)
    d, band = d.cpu().numpy(), band.cpu().numpy()
    assert band[np.abs(exact) < narrow - 0.05 * dx].all()
    assert not band[np.abs(exact) > narrow + 0.05 * dx].any()
    # chord error of the piecewise-linear section: about dx^2 / (8 radius)
    assert np.abs(d - exact)[band].max() < 0.02 * dx
    assert np.array_equal(d[~band], phi[~band])


def test_reinitialise_level_set_in_place():
    from pyaxisymflow_gb300.kernels.level_set import distance, reinitialise_level_set
    name, phi, dx = list(_fields())[0]
    t = torch.tensor(phi, device="cuda")
    d, _ = distance(t, dx, 5 * dx)
    reinitialise_level_set(t, dx, 5 * dx)
    assert torch.equal(t, d)
    with pytest.raises(ValueError):
        distance(t, dx, 5 * dx, out=t)
