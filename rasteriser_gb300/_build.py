"""Builds librast.so (the CUDA kernels and the C ABI) in-tree for sm_103a.

Translation units are compiled in parallel and only when a source or header is newer than the
object. The kernels are compiled with -fmad=false, IEEE division and square root and no flush to
zero; the host code with -ffp-contract=off. Both decide bit-exact parity with the reference.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIB_DIR, "librast.so")


def lib_path(checked=False):
    return os.path.join(LIB_DIR, "librast_checked.so" if checked else "librast.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build librast")
    return cand


def _units(checked=False):
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(PKG, "compat")]
    host = ["-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-std=c++17", "-O3"]
    kern = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
                   "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v"]
    if checked:
        kern = kern + ["-DRAST_CHECKED"]
    return [
        ("rast_kernels.cu", kern + inc),
        ("rast_shade.cu", kern + inc),
        ("rast_view.cu", kern + inc),
        ("rast_noalloc.cu", kern + inc),
        ("rast_api.cpp", host + inc),
        ("rast_batch.cpp", host + inc),
        ("rast_mlp.cpp", host + inc),
        ("rast_io.cpp", host + inc),
        ("rast_host_math.cpp", host + inc),
    ]


def _headers():
    hs = [os.path.join(ROOT, "include", "rast.h")]
    for d, _, fs in os.walk(CSRC):
        hs += [os.path.join(d, f) for f in fs if f.endswith((".h", ".cuh"))]
    for d, _, fs in os.walk(os.path.join(PKG, "compat")):
        hs += [os.path.join(d, f) for f in fs]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, checked=False):
    """Compile librast.so (or, with checked, librast_checked.so, whose kernels bounds-check every
    derived index) if anything changed; returns its path."""
    nvcc = nvcc_path()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    headers = _headers()
    jobs, objs = [], []
    lib = lib_path(checked)
    for src, flags in _units(checked):
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + (".checked.o" if checked else ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, "-c", s, "-o", o] + flags)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        logs = list(ex.map(run, jobs))
    if verbose:
        for lg in logs:
            print(lg)
    if force or jobs or _stale(lib, objs):
        run([nvcc, "-shared", "-o", lib] + ARCH + objs + ["-Xcompiler", "-fPIC"])
    if not checked:
        cli_src = os.path.join(PKG, "cpp", "rast_render.cpp")
        cli = cli_path()
        if force or _stale(cli, [cli_src, lib, os.path.join(ROOT, "include", "rast.h")]):
            cxx = shutil.which("g++") or "c++"
            run([cxx, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), cli_src, "-o", cli,
                 "-L" + LIB_DIR, "-lrast", "-Wl,-rpath,$ORIGIN"])
    return lib


def cli_path():
    """The headless renderer rast_render (rasteriser_gb300/cpp/rast_render.cpp)."""
    return os.path.join(LIB_DIR, "rast_render")


if __name__ == "__main__":
    import sys
    print(build(verbose=True, checked="--checked" in sys.argv))
