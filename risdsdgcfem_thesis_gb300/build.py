"""Build of the in-tree CUDA library libfemtet_gb300.so (sm_103a only).

Compiles every translation unit under csrc/ (.cu, and the host-only .cpp)
with nvcc in parallel and links
one shared library next to this file. rotation.cu is compiled without fused
multiply-adds so the FP64 rotation keeps the reference's rounding sequence.

A build is reused only when a stamp beside the library holds the same key:
a hash of every source and header, the compile and link flags, this file
and `nvcc --version` (so a changed flag, compiler or a library copied in
with a fresh modification time is rebuilt).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libfemtet_gb300.so")
BUILD_DIR = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I", os.path.join(HERE, "..", "include")]
PER_FILE = {"rotation.cu": ["--fmad=false"]}
LINK = ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def build_key(nv: str, defines=()) -> str:
    """Hash of everything the library is built from."""
    h = hashlib.sha256()
    deps = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC))
    deps += [os.path.join(HERE, "..", "include", "fem_tet.h"), os.path.abspath(__file__)]
    for p in deps:
        h.update(os.path.basename(p).encode())
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(repr((ARCH, COMMON, PER_FILE, LINK, tuple(defines))).encode())
    ver = subprocess.run([nv, "--version"], capture_output=True, text=True).stdout
    h.update(ver.encode())
    return h.hexdigest()


def build(verbose: bool = False, defines=(), out: str = OUT) -> str:
    """Builds the library (`defines`: extra -D flags, for a variant built
    to another `out` path) unless the stamp beside `out` matches."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    nv = nvcc()
    srcs = sources()
    key = build_key(nv, defines)
    stamp = out + ".key"
    if os.path.exists(out) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == key:
                return out
    tag = hashlib.sha256(repr(tuple(defines)).encode()).hexdigest()[:8] if defines else ""
    obj_dir = os.path.join(BUILD_DIR, tag) if tag else BUILD_DIR
    os.makedirs(obj_dir, exist_ok=True)
    dflags = [f"-D{d}" for d in defines]

    def compile_one(src):
        obj = os.path.join(obj_dir, os.path.splitext(src)[0] + ".o")
        cmd = [nv, *ARCH, *COMMON, *dflags, *PER_FILE.get(src, []), "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = out + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, *LINK]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    with open(stamp, "w") as f:
        f.write(key + "\n")
    return out


BOUNDS_OUT = os.path.join(HERE, "libfemtet_gb300_bounds.so")


def build_bounds_check(verbose: bool = False) -> str:
    """The diagnostic variant: every table-read index in the kernels checked
    against its limit (bounds.cuh), libfemtet_gb300_bounds.so."""
    return build(verbose=verbose, defines=("FEM_BOUNDS_CHECK",), out=BOUNDS_OUT)


if __name__ == "__main__":
    print(build(verbose=True))
