"""Build recipe of the oracle's native parts (test infrastructure only).

* oracle/_ref/libref_lsq.so: the reference's own least-squares core compiled
  from its sources in place (core/src/extrapolate_using_least_squares.hpp)
  through oracle/ref_shim.cpp.
* oracle/_ref/libref_p2m.so: the reference's particle-to-mesh and
  mesh-to-particle interpolation (core/src/particles_to_mesh.hpp,
  core/src/mesh_to_particles.hpp) through oracle/ref_p2m_shim.cpp.
Built only where the reference sources exist; never shipped.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("PYAXISYMFLOW_REF", "/root/reference")
REF_DIR = os.path.join(HERE, "_ref")


def ref_lsq_path():
    return os.path.join(REF_DIR, "libref_lsq.so")


def ref_p2m_path():
    return os.path.join(REF_DIR, "libref_p2m.so")


def _build_shim(shim_name, out):
    src_dir = os.path.join(REF_ROOT, "pyaxisymflow", "core", "src")
    if not os.path.isdir(src_dir):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    shim = os.path.join(HERE, shim_name)
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(shim):
        return out
    # no FMA contraction: the reference's expressions evaluated as written
    cmd = ["g++", "-O2", "-std=c++14", "-fPIC", "-shared", "-ffp-contract=off", "-I", src_dir,
           "-o", out, shim]
    subprocess.run(cmd, check=True)
    return out


def build_ref():
    return _build_shim("ref_shim.cpp", ref_lsq_path())


def build_ref_p2m():
    return _build_shim("ref_p2m_shim.cpp", ref_p2m_path())


def build_all():
    return {"ref_lsq": build_ref(), "ref_p2m": build_ref_p2m()}


if __name__ == "__main__":
    print(build_all())
