"""In-tree build of the sm_103a rasterizer library (libifrit_gb300.so).

Compiles the CUDA translation units in parallel with nvcc for sm_103a only and links one
shared library next to this file.  --fmad=false keeps every float expression in the exact
evaluation order the CPU checker uses (no contraction into FMA).
"""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libifrit_gb300.so")
SOURCES = ["raster_kernels.cu", "capi.cu", "noalloc.cu", "diff_kernels.cu"]
HEADERS = ["raster_math.cuh", "raster_kernels.cuh", "pass_plan.h", os.path.join("..", "..", "include", "ifrit_gb300.h")]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
FLAGS = ["-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "--fmad=false",
         "-Xcompiler", "-fPIC,-fvisibility=hidden", "-Xptxas", "-v"]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.abspath(__file__)]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(BUILD, src + ".o")
        cmd = [NVCC] + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-6000:]))
        with open(os.path.join(BUILD, src + ".ptxas.txt"), "w") as f:
            f.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [NVCC, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


INCLUDE = os.path.join(os.path.dirname(ROOT), "include")


def build_extension(sources, out, extra_flags=()):
    """Compiles CUDA sources written against the device-side extension point
    (include/ifrit_gb300_ext.cuh: shading functors, mesh-stage functors) into the shared library
    `out`, for sm_103a with the library's own float flags, linked against libifrit_gb300.so."""
    build()
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    tmp = out + ".tmp"
    flags = ["-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "--fmad=false",
             "-Xcompiler", "-fPIC"]
    cmd = ([NVCC] + flags + ["-shared", "-I", INCLUDE] +
           list(extra_flags) + list(sources) + ["-o", tmp, "-L", PKG, "-lifrit_gb300", "-Xlinker", "-rpath," + PKG])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("extension build failed:\n" + r.stderr[-6000:])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    build(force=True, verbose=True)
