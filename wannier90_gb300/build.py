"""Build recipe of the in-tree CUDA library ``wannier90_gb300/lib/libw90gb300.so``.

Compiles the CUDA translation units for sm_103a only (GB300) and the host C++ units,
in parallel, then links one shared library with the static CUDA runtime.  No cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIBNAME = "libw90gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _nvcc():
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build wannier90_gb300")
    return p


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, extra_nvcc=(), libdir=None):
    """Compile and link; returns the library path.  libdir / extra_nvcc give a separate
    build (e.g. the bounded-wait test's, with -DW90G_SPIN_LIMIT=...) beside the main one."""
    nvcc = _nvcc()
    libdir = libdir or LIBDIR
    os.makedirs(os.path.join(libdir, "obj"), exist_ok=True)
    cu, cpp = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "wannier90_gb300.h"))
    jobs = []
    objs = []
    for f in cu + cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(libdir, "obj", f + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [src] + headers):
            continue
        if f.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xptxas", "-v" if verbose else "-O3", *extra_nvcc, "-c", src, "-o", obj]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-I" + os.path.join(CUDA_HOME, "include"),
                   "-c", src, "-o", obj]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(run, jobs))
    for cmd, r in results:
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    out = os.path.join(libdir, LIBNAME)
    if force or _stale(out, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", out, *objs, "-lcudart_static" if False else "-cudart=static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
