"""The C-ABI library builds, loads without a GPU and exports every declared symbol."""
import ctypes
import os
import re

from pyaxisymflow_gb300 import build as gbuild

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(REPO, "include", "axisym_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(axi_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    path = gbuild.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from pyaxisymflow_gb300 import _native
    assert set(declared_symbols()) <= set(_native.SIGNATURES)
    lib = _native.lib()
    assert lib.axi_version() >= 100
    assert lib.axi_last_error() == b""


def test_no_cpu_fallback_for_cpu_tensors():
    import pytest
    import torch

    from pyaxisymflow_gb300.kernels.brinkmann_penalize import brinkmann_penalize
    t = torch.zeros((4, 4), dtype=torch.float64)
    with pytest.raises(ValueError, match="CUDA"):
        brinkmann_penalize(1.0, 1.0, t, 0.0, 0.0, t, t, t, t)


def test_new_entry_points_reject_bad_arguments_before_any_launch():
    """Argument checks of the particle, mesh-to-particle and level-set entry
    points run on the host before anything touches the GPU: null pointers,
    bad sizes and aliasing come back as AXI_ERR_INVALID with a message naming
    the call (fake non-null pointers are never dereferenced)."""
    import ctypes as c

    from pyaxisymflow_gb300 import _native as N
    lib = N.lib()
    P = c.c_void_p
    fake = P(4096)  # never dereferenced: every call below fails its checks first
    null = P(None)

    st = lib.axi_level_set_distance_f64(null, fake, 8, 8, 0.1, 0.5, null, fake, null)
    assert st == N.AXI_ERR_INVALID and b"level_set_distance" in lib.axi_last_error()
    st = lib.axi_level_set_distance_f64(fake, fake, 8, 8, 0.1, 0.5, null, fake, null)
    assert st == N.AXI_ERR_INVALID and b"alias" in lib.axi_last_error()
    st = lib.axi_level_set_distance_f64(P(8192), fake, 8, 8, 0.0, 0.5, null, fake, null)
    assert st == N.AXI_ERR_INVALID
    st = lib.axi_level_set_distance_f64(P(8192), fake, 1, 8, 0.1, 0.5, null, fake, null)
    assert st == N.AXI_ERR_INVALID
    assert lib.axi_level_set_work_bytes(1, 8) == 0 and lib.axi_level_set_work_bytes(8, 8) > 0

    st = lib.axi_mesh_to_particles_2d_mp4_f64(fake, fake, 0, 8, fake, fake, fake, fake, 4, 4,
                                              0.1, 0.1, 1, null)
    assert st == N.AXI_ERR_INVALID and b"mesh_to_particles" in lib.axi_last_error()
    st = lib.axi_mesh_to_particles_2d_mp4_f64(fake, null, 8, 8, fake, fake, fake, fake, 4, 4,
                                              0.1, 0.1, 1, null)
    assert st == N.AXI_ERR_INVALID

    st = lib.axi_particles_to_mesh_2d_mp4_f64(fake, fake, fake, fake, 4, 8, 0.1, 0.1, 0, fake,
                                              null)
    assert st == N.AXI_ERR_INVALID and b"particles_to_mesh" in lib.axi_last_error()
    assert lib.axi_p2m_mp4_work_bytes(0, 8) == 0


def test_spectral_transforms_reject_null_fields():
    """Both FP64 spectral transform entry points (with caller scratch and with
    the library's static scratch) reject null input and output pointers on the
    host, before any launch."""
    import ctypes as c

    from pyaxisymflow_gb300 import _native as N
    lib = N.lib()
    fake, null = c.c_void_p(4096), c.c_void_p(None)
    for out, inp in ((null, fake), (fake, null)):
        st = lib.axi_fd_transform_f64(out, 8, inp, 8, fake, fake, fake, fake, fake, fake, 8, 8,
                                      null)
        assert st == N.AXI_ERR_INVALID and b"fd_transform" in lib.axi_last_error()
        st = lib.axi_fd_transform_static_f64(out, 8, inp, 8, fake, fake, fake, fake, fake, 8, 8,
                                             null)
        assert st == N.AXI_ERR_INVALID and b"fd_transform_static" in lib.axi_last_error()


def test_soft_loop_entries_reject_null_pointers():
    """Every pointer argument of the device-resident soft-loop entries is
    checked on the host: a null one comes back as AXI_ERR_INVALID naming the
    argument, before any launch (the stream argument, last, may be null)."""
    import ctypes as c

    from pyaxisymflow_gb300 import _native as N
    lib = N.lib()
    F = 4096  # fake non-null device address, never dereferenced
    n, nr, nz = 64, 8, 8
    # (entry, arguments with fake pointers as "P", positions of the pointers checked)
    calls = {
        "axi_soft_dt_f64": ["P", "P", n, "P", 1.0, 0.1, 1.0, 1e-10, None],
        "axi_soft_advect_eno3_f64": ["P", "P", 1, "P", "P", "P", nr, nz, 0.1, "P", None],
        "axi_soft_pin_level_set_f64": ["P", "P", "P", n, 0.5, 0.1, 0.05, None],
        "axi_soft_mask_f64": ["P", "P", "P", n, 0.01, None],
        "axi_soft_extrapolate_eta_f64": ["P", "P", "P", "P", "P", "P", "P", "P", "P", 0.1, nr, nz,
                                         "P", "P", 10, "P", "P", None],
        "axi_soft_stress_mask_f64": ["P", "P", "P", "P", n, None],
        "axi_soft_update_vorticity_from_solid_stress_f64": ["P", "P", "P", "P", "P", "P", "P", nr,
                                                            nz, 0.1, "P", None],
        "axi_soft_tether_f64": ["P", "P", "P", n, "P", 0.5, 0.1, 6.28, 0.1, 0.01, None],
        "axi_soft_penalise_f64": ["P", "P", "P", "P", "P", "P", nr, nz, 0.1, 1e6, 0.1, 6.28, "P",
                                  None],
        "axi_soft_diffusion_rk2_f64": ["P", "P", "P", nr, nz, 0.01, 0.1, "P", None],
        "axi_soft_advance_f64": ["P", None],
    }
    for name, proto in calls.items():
        fn = getattr(lib, name)
        ptrs = [q for q, a in enumerate(proto) if a == "P"]
        assert ptrs, name
        for q in ptrs:
            args = [c.c_void_p(F) if a == "P" else (c.c_void_p(None) if a is None else a)
                    for a in proto]
            args[q] = c.c_void_p(None)
            st = fn(*args)
            assert st == N.AXI_ERR_INVALID, (name, q, st)
            msg = lib.axi_last_error()
            assert b"null" in msg and name[4:-4].encode() in msg, (name, q, msg)


def test_drop_in_entries_reject_null_pointers():
    """The drop-in kernel entries (both precisions) check their field pointers
    on the host too: with any one of them null the call returns
    AXI_ERR_INVALID naming it, before any launch."""
    import ctypes as c

    from pyaxisymflow_gb300 import _native as N
    lib = N.lib()
    F = 4096  # fake non-null device address, never dereferenced
    nr = nz = 16
    n = nr * nz
    for s in ("f64", "f32"):
        calls = {
            f"axi_velocity_from_psi_unb_{s}": ["P", "P", "P", "P", nr, nz, 0.1, None],
            f"axi_velocity_from_psi_periodic_{s}": ["P", "P", "P", "P", nr, nz, 0.1, 1, None],
            f"axi_vorticity_from_velocity_unb_{s}": ["P", "P", "P", nr, nz, 0.1, None],
            f"axi_vorticity_from_velocity_periodic_{s}": ["P", "P", "P", nr, nz, 0.1, 1, None],
            f"axi_brinkmann_penalize_{s}": [1e4, 0.01, "P", 0.0, 0.0, "P", "P", "P", "P", n, None],
            f"axi_smooth_heaviside_{s}": ["P", "P", 0.1, n, None],
            f"axi_kill_boundary_vorticity_sine_z_{s}": ["P", "P", nr, nz, 3, 0.1, None],
            f"axi_kill_boundary_vorticity_sine_r_{s}": ["P", "P", nr, nz, 3, 0.1, None],
            f"axi_diffusion_rk2_unb_{s}": ["P", "P", "P", nr, nz, 0.01, 0.01, 0.1, None],
            f"axi_diffusion_rk2_periodic_{s}": ["P", "P", "P", nr, nz, 0.01, 0.01, 0.1, 1, None],
            f"axi_periodic_ghost_comm_{s}": ["P", nr, nz, 1, None],
            f"axi_compute_force_on_body_{s}": ["P", "P", 1.0, 1e4, "P", 0.0, 1.0, 0.01, 0.0, n,
                                               "P", "P", None],
            f"axi_force_projection_{s}": [1.0, "P", "P", "P", "P", n, "P", "P", None],
            f"axi_advect_vorticity_eno3_{s}": ["P", "P", "P", "P", nr, nz, 0.1, None],
            f"axi_advect_refmap_eno3_{s}": ["P", "P", "P", "P", "P", nr, nz, 0.1, None],
            f"axi_solid_sigma_{s}": ["P", "P", "P", 1e-3, 0.1, "P", "P", "P", "P", "P", "P", nr,
                                     nz, None],
            f"axi_update_vorticity_from_solid_stress_{s}": ["P", "P", "P", "P", "P", "P", "P", nr,
                                                            nz, 0.01, 0.1, None],
        }
        if s == "f64":
            calls["axi_extrapolate_lsq_first_order_f64"] = ["P", "P", "P", "P", "P", "P", nr, nz,
                                                            10, "P", None, None]
            calls["axi_extrapolate_eta_with_least_squares_f64"] = [
                "P", "P", "P", "P", "P", "P", "P", "P", "P", 0.1, nr, nz, "P", "P", 10, "P", None,
                None]
        for name, proto in calls.items():
            fn = getattr(lib, name)
            for q in [q for q, a in enumerate(proto) if a == "P"]:
                args = [c.c_void_p(F) if a == "P" else (c.c_void_p(None) if a is None else a)
                        for a in proto]
                args[q] = c.c_void_p(None)
                st = fn(*args)
                assert st == N.AXI_ERR_INVALID, (name, q, st)
                assert b"null" in lib.axi_last_error(), (name, q, lib.axi_last_error())
