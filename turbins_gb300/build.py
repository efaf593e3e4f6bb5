"""Build recipe of libturbgpu.so: every CUDA source under csrc/ is compiled for
sm_103a only (one -gencode), in parallel, and linked into an in-tree shared
library next to this file (turbins_gb300/lib/).  libturbdropin.so, the layer
that takes the reference's own routine names (dropin/turbins_dropin.c), is
compiled with gcc beside it and linked to libturbgpu.so; its PETSc vector
calls resolve in the host program."""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
LIB = os.path.join(OUT, "libturbgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
           "--expt-relaxed-constexpr", "-Xptxas", "-O3"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _compile(src, obj, verbose):
    cmd = [nvcc()] + ARCH + NVFLAGS + (["-Xptxas", "-v"] if verbose else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return r.stderr


DROPIN_SRC = os.path.join(HERE, "dropin", "turbins_dropin.c")
DROPIN = os.path.join(OUT, "libturbdropin.so")


def build_dropin(force=False):
    deps = [DROPIN_SRC, LIB, os.path.join(HERE, "..", "include", "turbins_dropin.h")]
    if not force and os.path.exists(DROPIN) and all(os.path.getmtime(d) <= os.path.getmtime(DROPIN) for d in deps):
        return DROPIN
    tmp = DROPIN + ".tmp"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-Wall", "-o", tmp, DROPIN_SRC, "-L" + OUT, "-lturbgpu",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("drop-in layer build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, DROPIN)
    return DROPIN


def build(force=False, verbose=False):
    lib = _build_gpu(force, verbose)
    build_dropin(force)
    return lib


def _build_gpu(force=False, verbose=False):
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    deps = srcs + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(HERE, "..", "include", "turbins_gb300.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= t for s in deps if os.path.exists(s)):
            return LIB
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    objs = [os.path.join(objdir, os.path.basename(s)[:-3] + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        logs = list(ex.map(lambda a: _compile(a[0], a[1], verbose), zip(srcs, objs)))
    if verbose:
        for s, lg in zip(srcs, logs):
            print("==", os.path.basename(s))
            print(lg)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
