"""Build recipe of the CUDA library behind include/axisym_gb300.h.

Compiles every ``csrc/*.cu`` translation unit for sm_103a only, in parallel,
and links ``_build/libaxisym_gb300.so`` in-tree. No cmake; nvcc only.
"""
import concurrent.futures
import hashlib
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libaxisym_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(home, "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def lib_path():
    return os.path.join(OUT_DIR, LIB_NAME)


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _inputs_digest():
    h = hashlib.sha256()
    files = _sources() + sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                                if f.endswith((".cuh", ".h")))
    files.append(os.path.join(REPO, "include", "axisym_gb300.h"))
    for f in files:
        with open(f, "rb") as fh:
            h.update(f.encode())
            h.update(fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compile and link the library if any source changed; return its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    stamp = os.path.join(OUT_DIR, "stamp.txt")
    digest = _inputs_digest()
    if not force and os.path.exists(lib_path()) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return lib_path()
    srcs = _sources()
    objs = [os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-I", os.path.join(REPO, "include"), "-c", src,
                                              "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    workers = max(1, min(len(srcs), os.cpu_count() or 4))
    with concurrent.futures.ThreadPoolExecutor(workers) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    tmp = lib_path() + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path())
    with open(stamp, "w") as f:
        f.write(digest)
    return lib_path()


if __name__ == "__main__":
    print(build(force=True, verbose=True))
