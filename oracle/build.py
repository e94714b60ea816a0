"""Build recipe of the oracle's native parts (test infrastructure only).

* oracle/_ref/libref_lsq.so: the reference's own least-squares core compiled
  from its sources in place (core/src/extrapolate_using_least_squares.hpp)
  through oracle/ref_shim.cpp. Built only where the reference sources exist.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("PYAXISYMFLOW_REF", "/root/reference")
REF_DIR = os.path.join(HERE, "_ref")


def ref_lsq_path():
    return os.path.join(REF_DIR, "libref_lsq.so")


def build_ref():
    src_dir = os.path.join(REF_ROOT, "pyaxisymflow", "core", "src")
    if not os.path.isdir(src_dir):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    out = ref_lsq_path()
    shim = os.path.join(HERE, "ref_shim.cpp")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(shim):
        return out
    cmd = ["g++", "-O2", "-std=c++14", "-fPIC", "-shared", "-ffp-contract=off", "-I", src_dir,
           "-o", out, shim]
    subprocess.run(cmd, check=True)
    return out


def build_all():
    return {"ref_lsq": build_ref()}


if __name__ == "__main__":
    print(build_all())
