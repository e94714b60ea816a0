"""Output utilities on the host: the VTK image writer (interface of the
reference's utils/dump_vtk.py) and the ensemble snapshot file format."""
import numpy as np
import pytest


def test_vtk_write_round_trip(tmp_path):
    from pyaxisymflow_gb300.utils.dump_vtk import read_vti, vtk_init, vtk_write
    nz, nr = 24, 10
    rng = np.random.default_rng(0)
    fields = [rng.standard_normal((nr, nz)) for _ in range(3)]
    names = ["vorticity", "psi", "char_func"]
    img, arr, writer = vtk_init(nz, nr)
    path = tmp_path / "fields.vti"
    vtk_write(str(path), img, arr, writer, names, fields, nz, nr)
    back = read_vti(str(path))
    assert back["_dims"] == (nz, nr) and back["_name"] == "softy"
    for n, f in zip(names, fields):
        assert np.array_equal(back[n], f)
    # the writer is reusable, as the reference drivers call it every few steps
    vtk_write(str(path), img, arr, writer, ["a"], [fields[0] * 2], nz, nr)
    assert np.array_equal(read_vti(str(path))["a"], fields[0] * 2)


def test_vtk_write_checks_sizes(tmp_path):
    from pyaxisymflow_gb300.utils.dump_vtk import vtk_init, vtk_write
    img, arr, writer = vtk_init(8, 4)
    with pytest.raises(ValueError):
        vtk_write(str(tmp_path / "x.vti"), img, arr, writer, ["a"], [np.zeros((4, 7))], 8, 4)
    with pytest.raises(ValueError):
        vtk_write(str(tmp_path / "x.vti"), img, arr, writer, ["a", "b"], [np.zeros((4, 8))], 8, 4)


def test_snapshot_file_round_trip(tmp_path):
    import dataclasses

    from pyaxisymflow_gb300.engine import ST_WORDS, RigidBodyCase
    from pyaxisymflow_gb300.utils.snapshot import FIELDS, read_snapshot, write_snapshot
    rng = np.random.default_rng(1)
    cases = [RigidBodyCase(nz=64, nr=32, dx=2.0 / 64, seed=3),
             RigidBodyCase(nz=96, nr=48, dx=2.0 / 96, sediment=True, U0=0.0, ramp=False)]
    snap = {
        "format": "pyaxisymflow-gb300 rigid ensemble snapshot 1", "precision": "f32",
        "tensor_cores": True, "dct": True,
        "cases": [dataclasses.asdict(c) for c in cases],
        "state": rng.standard_normal((2, ST_WORDS)),
        "fields": [{n: rng.standard_normal((c.nr, c.nz)).astype(np.float32) for n in FIELDS}
                   for c in cases],
        "history": [rng.standard_normal((5, 2)), rng.standard_normal((5, 2))],
    }
    path = tmp_path / "snap.npz"
    write_snapshot(str(path), snap)
    back = read_snapshot(str(path))
    assert [RigidBodyCase(**c) for c in back["cases"]] == cases
    assert back["precision"] == "f32" and back["dct"] and back["tensor_cores"]
    assert np.array_equal(back["state"], snap["state"])
    for a, b in zip(back["fields"], snap["fields"]):
        for n in FIELDS:
            assert a[n].dtype == b[n].dtype and np.array_equal(a[n], b[n])
    for a, b in zip(back["history"], snap["history"]):
        assert np.array_equal(a, b)
    np.savez(str(tmp_path / "other.npz"), meta=np.array('{"format": "x"}'))
    with pytest.raises(ValueError):
        read_snapshot(str(tmp_path / "other.npz"))
