"""Build recipe of the oracle's native parts (test infrastructure only).

* oracle/_ref/libref_lsq.so: the reference's own least-squares core compiled
  from its sources in place (core/src/extrapolate_using_least_squares.hpp)
  through oracle/ref_shim.cpp.
* oracle/_ref/libref_p2m.so: the reference's particle-to-mesh and
  mesh-to-particle interpolation (core/src/particles_to_mesh.hpp,
  core/src/mesh_to_particles.hpp) through oracle/ref_p2m_shim.cpp.
Built only where the reference sources exist (their root is given by the
caller or by the PYAXISYMFLOW_REF environment variable); never shipped.
* oracle/_build/libora_step.so: the oracle's own C restatement of the
  per-step grid kernels (oracle/cstep.c, OpenMP), the timed CPU baseline;
  built everywhere.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
BUILD_DIR = os.path.join(HERE, "_build")


def ref_lsq_path():
    return os.path.join(REF_DIR, "libref_lsq.so")


def ref_p2m_path():
    return os.path.join(REF_DIR, "libref_p2m.so")


def _ref_root(ref_root):
    return ref_root if ref_root else os.environ.get("PYAXISYMFLOW_REF")


def _build_shim(shim_name, out, ref_root):
    if not ref_root:
        return None
    src_dir = os.path.join(ref_root, "pyaxisymflow", "core", "src")
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


def build_ref(ref_root=None):
    return _build_shim("ref_shim.cpp", ref_lsq_path(), _ref_root(ref_root))


def build_ref_p2m(ref_root=None):
    return _build_shim("ref_p2m_shim.cpp", ref_p2m_path(), _ref_root(ref_root))


def cstep_path():
    return os.path.join(BUILD_DIR, "libora_step.so")


def build_cstep():
    """Compiles oracle/cstep.c (portable flags: no -march, no FMA contraction,
    so it gives the numpy oracle's bits on x86 and Arm alike)."""
    src = os.path.join(HERE, "cstep.c")
    out = cstep_path()
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = out + ".tmp"
    subprocess.run(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                    "-o", tmp, src, "-lm"], check=True)
    os.replace(tmp, out)
    return out


def build_all(ref_root=None):
    """Builds the oracle's C restatement and what the given reference root (or
    PYAXISYMFLOW_REF) allows of the reference's own sources."""
    return {"cstep": build_cstep(), "ref_lsq": build_ref(ref_root),
            "ref_p2m": build_ref_p2m(ref_root)}


if __name__ == "__main__":
    import sys
    print(build_all(sys.argv[1] if len(sys.argv) > 1 else None))
