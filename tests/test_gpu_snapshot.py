"""Checkpoint / restore of the engine: a restored ensemble continues
bit-identically, and fields written to VTK match the device fields."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _cases():
    from pyaxisymflow_gb300.engine import RigidBodyCase
    return [RigidBodyCase(nz=128, nr=64, dx=2.0 / 128, r_sphere=0.1, seed=5),
            RigidBodyCase(nz=192, nr=96, dx=2.0 / 192, r_sphere=0.08, z_cm=1.2, U0=0.0,
                          ramp=False, sediment=True, rho_s=2.0, seed=6)]


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_restored_ensemble_continues_bit_identically(tmp_path, precision):
    from pyaxisymflow_gb300.engine import RigidEnsemble
    from pyaxisymflow_gb300.utils.snapshot import load_checkpoint, save_checkpoint
    ens = RigidEnsemble(_cases(), precision=precision, history_steps=40)
    ens.step(12)
    path = str(tmp_path / "ck.npz")
    save_checkpoint(ens, path)
    ens.step(9)
    back = load_checkpoint(path)
    assert back.precision == precision and back.dct == ens.dct
    back.step(9)
    torch.cuda.synchronize()
    assert not ens.status().any() and not back.status().any()
    assert torch.equal(back.state, ens.state)
    assert torch.equal(back.history, ens.history)
    for a, b in zip(back.fields, ens.fields):
        for n in ("omega", "psi", "u_z", "u_r", "chi"):
            assert torch.equal(a[n], b[n]), n


def test_vtk_output_of_device_fields(tmp_path):
    from pyaxisymflow_gb300.engine import RigidEnsemble
    from pyaxisymflow_gb300.utils.dump_vtk import read_vti, vtk_init, vtk_write
    c = _cases()[0]
    ens = RigidEnsemble([c], precision="f32")
    ens.step(3)
    f = ens.fields[0]
    img, arr, writer = vtk_init(c.nz, c.nr)
    path = str(tmp_path / "out.vti")
    vtk_write(path, img, arr, writer, ["vorticity", "psi"], [f["omega"], f["psi"]], c.nz, c.nr)
    back = read_vti(path)
    assert np.array_equal(back["vorticity"], f["omega"].double().cpu().numpy())
    assert np.array_equal(back["psi"], f["psi"].double().cpu().numpy())
