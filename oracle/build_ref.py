"""Build recipe for the reference's own CPU code (test infrastructure only).

Two things are built from the reference checkout named by the environment variable
IFRIT_REFERENCE_ROOT (there is no default location):

* the reference CPU tile rasterizer (TileRasterRenderer and its worker, 8 source files)
  together with ``oracle/ref_driver.cpp`` into ``oracle/_ref/libifrit_ref.so``;
* the reference texture sampler (the host-compilable ``TextureSampleImpl`` functions of
  include/ifrit/softgraphics/engine/math/ShaderBuiltinCuda.cuh:96-272) together with
  ``oracle/ref_sampler.cu`` into ``oracle/_ref/libifrit_ref_sampler.so`` (nvcc, host code only).

Everything goes into the git-ignored ``oracle/_ref/``; nothing from the reference is committed.
The renderer is built from a staged tree, ``oracle/_ref/src/``: ``stage()`` copies the 8 sources
and exactly the headers they include (as ``g++ -MM`` lists them) there and applies the overlays
below by pattern, so the same staged tree can be compiled on another host (the GPU host is an
Arm machine with no reference checkout; the staged tree travels with the working copy there,
never into the repository's history).  Overlays:

* ``ifrit/core/typing/Util.h``: the dead ``#ifdef __PRETTY_FUNCTION__`` branch ending in
  ``static_assert(false)`` (include/ifrit/core/typing/Util.h:113-124) is rejected by GCC 13;
  the overlay keeps only the ``__PRETTY_FUNCTION__`` return.
* ``ifrit/softgraphics/engine/tileraster/TileRasterContext.h``: ``numThreads`` (a compile-time
  constant, 16 in the reference, TileRasterContext.h:52) becomes ``IFRIT_REF_NUM_THREADS``, set
  at compile time to the host's core count minus one, because the reference's spin barriers
  degrade sharply when oversubscribed.
* ``ifrit/core/platform/ApiConv.h``: the 64-bit platform test (``ApiConv.h:69``) knows x86-64
  and ppc64 only and fails a ``static_assert`` elsewhere; the overlay adds aarch64.
* Scalar build (``simd=False``, the only build on a non-x86 host): the three x86 intrinsic sites
  that the reference uses even with its SIMD switches off are put under the switches:
  ``Image.h:110-113`` (``fillPixelRGBA128ps``, only called from SIMD-128 code) and the
  ``_mm256_set1_epi32`` constants of ``TileRasterWorker.cpp:1689-1690, 1938-1939`` (only used by
  SIMD-256 code); and the scalar branch of ``pixelShadingFromTagBuffer`` calls ``dot``, a name
  the vector library spells ``Dot`` (``TileRasterWorker.cpp:2099-2100``, compiled only without
  SIMD).  The x86 build keeps the reference's AVX2 flags.
"""
import os
import platform
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(OUT, "src")
REF_ROOT = os.environ.get("IFRIT_REFERENCE_ROOT")

SOURCES = [
    "projects/softgraphics/src/engine/tileraster/TileRasterRenderer.cpp",
    "projects/softgraphics/src/engine/tileraster/TileRasterWorker.cpp",
    "projects/softgraphics/src/engine/base/FrameBuffer.cpp",
    "projects/softgraphics/src/engine/base/TypeDescriptor.cpp",
    "projects/softgraphics/src/engine/base/VaryingDescriptor.cpp",
    "projects/softgraphics/src/engine/base/VertexBuffer.cpp",
    "projects/softgraphics/src/engine/base/VertexShaderResult.cpp",
    "projects/softgraphics/src/engine/bufferman/BufferManager.cpp",
]

COMMON = ["-std=c++20", "-O2", "-fPIC", "-DIFRIT_DLL", "-DIFRIT_API_EXPORT", "-w"]
SIMD_FLAGS = ["-mavx2", "-mfma", "-DIFRIT_FEATURE_SIMD=1", "-DIFRIT_FEATURE_SIMD_AVX256=1"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


def is_x86():
    return platform.machine() in ("x86_64", "AMD64")


def have_checkout():
    return bool(REF_ROOT) and os.path.isdir(REF_ROOT)


def staged():
    return os.path.exists(os.path.join(STAGE, "STAGED"))


def available():
    """True if the renderer can be built here (a staged tree or a checkout to stage from)."""
    return staged() or have_checkout()


def _overlay(rel, text):
    """Applies the overlays to one staged file's text."""
    if rel == "include/ifrit/core/typing/Util.h":
        pat = re.compile(r"#ifdef __PRETTY_FUNCTION__\s*return __PRETTY_FUNCTION__;\s*#else\s*"
                         r"static_assert\(false, \"Unsupported compiler\"\);\s*#endif")
        text, n = pat.subn("return __PRETTY_FUNCTION__;", text)
        if n != 1:
            raise RuntimeError("Util.h overlay pattern not found")
    elif rel == "include/ifrit/softgraphics/engine/tileraster/TileRasterContext.h":
        text, n = re.subn(r"(IF_CONSTEXPR static int numThreads\s*=\s*)16;", r"\g<1>IFRIT_REF_NUM_THREADS;", text)
        if n != 1:
            raise RuntimeError("TileRasterContext.h overlay pattern not found")
    elif rel == "include/ifrit/core/platform/ApiConv.h":
        text, n = re.subn(r"#if __x86_64__ \|\| __ppc64__", "#if __x86_64__ || __ppc64__ || __aarch64__", text)
        if n != 1:
            raise RuntimeError("ApiConv.h overlay pattern not found")
    elif rel == "include/ifrit/softgraphics/core/data/Image.h":
        pat = re.compile(r"(\n[ \t]*inline void fillPixelRGBA128ps\(size_t x, size_t y, const __m128& ps\)\s*"
                         r"\{[^{}]*\})")
        text, n = pat.subn(r"\n#ifdef IFRIT_USE_SIMD_128\1\n#endif", text)
        if n != 1:
            raise RuntimeError("Image.h overlay pattern not found")
    elif rel.endswith("tileraster/TileRasterWorker.cpp"):
        pat = re.compile(r"(\n[ \t]*auto\s+aCsFwS1\s*=\s*_mm256_set1_epi32\([^;]*\);\s*"
                         r"\n[ \t]*auto\s+aCsFhS1\s*=\s*_mm256_set1_epi32\([^;]*\);)")
        text, n = pat.subn(r"\n#ifdef IFRIT_USE_SIMD_256\1\n#endif", text)
        if n != 2:
            raise RuntimeError("TileRasterWorker.cpp overlay pattern found %d times" % n)
        text, n = re.subn(r"= dot\(baryVec, (atpB[xy])\);", r"= Dot(baryVec, \1);", text)
        if n != 2:
            raise RuntimeError("TileRasterWorker.cpp dot overlay found %d times" % n)
    return text


def stage():
    """Copies the renderer sources and the headers they include into oracle/_ref/src/ with
    the overlays applied.  Needs the checkout (IFRIT_REFERENCE_ROOT)."""
    if not have_checkout():
        raise RuntimeError("IFRIT_REFERENCE_ROOT does not name a reference checkout")
    inc = os.path.join(REF_ROOT, "include")
    srcs = [os.path.join(REF_ROOT, s) for s in SOURCES]
    # dependency list of the SIMD build (a superset of the scalar build's)
    r = subprocess.run(["g++", "-MM"] + COMMON + SIMD_FLAGS + ["-DIFRIT_REF_NUM_THREADS=1", "-I" + inc] + srcs,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("dependency scan failed:\n" + r.stderr[-4000:])
    deps = set()
    for tok in r.stdout.replace("\\\n", " ").split():
        if tok.endswith(":"):
            continue
        p = os.path.realpath(tok if os.path.isabs(tok) else os.path.join(os.getcwd(), tok))
        if p.startswith(os.path.realpath(REF_ROOT) + os.sep):
            deps.add(os.path.relpath(p, os.path.realpath(REF_ROOT)))
    if os.path.isdir(STAGE):
        shutil.rmtree(STAGE)
    for rel in sorted(deps):
        dst = os.path.join(STAGE, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        with open(os.path.join(REF_ROOT, rel), encoding="utf-8", errors="surrogateescape") as f:
            text = f.read()
        with open(dst, "w", encoding="utf-8", errors="surrogateescape") as f:
            f.write(_overlay(rel, text))
    with open(os.path.join(STAGE, "STAGED"), "w") as f:
        f.write("\n".join(sorted(deps)) + "\n")
    return STAGE


def build(num_threads=None, simd=None, quiet=True):
    """Compile the reference renderer + driver from the staged tree (staging it first when a
    checkout is available); returns the .so path or None.  simd=None: AVX2 build on x86,
    scalar build elsewhere."""
    if not available():
        return None
    if simd is None:
        simd = is_x86()
    if simd and not is_x86():
        raise RuntimeError("the SIMD build of the reference needs an x86 host")
    if num_threads is None:
        num_threads = max(1, (os.cpu_count() or 2) - 1)
    name = "libifrit_ref.so" if simd else "libifrit_ref_scalar.so"
    lib = os.path.join(OUT, name)
    stamp = lib + ".stamp"
    driver = os.path.join(HERE, "ref_driver.cpp")
    if not staged() or (have_checkout() and os.path.getmtime(os.path.join(STAGE, "STAGED")) < os.path.getmtime(__file__)):
        stage()
    key = "%d %d" % (num_threads, int(simd))
    if (os.path.exists(lib) and os.path.exists(stamp) and open(stamp).read().strip() == key
            and os.path.getmtime(lib) >= max(os.path.getmtime(driver), os.path.getmtime(os.path.join(STAGE, "STAGED")))):
        return lib
    objdir = os.path.join(OUT, "obj_simd" if simd else "obj_scalar")
    os.makedirs(objdir, exist_ok=True)
    flags = COMMON + (SIMD_FLAGS if simd else []) + ["-DIFRIT_REF_NUM_THREADS=%d" % num_threads,
                                                     "-I" + os.path.join(STAGE, "include")]
    jobs = []
    for src in [os.path.join(STAGE, s) for s in SOURCES] + [driver]:
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        jobs.append((["g++"] + flags + ["-c", src, "-o", obj], obj))

    def run(job):
        cmd, obj = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
        return obj

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(run, jobs))
    r = subprocess.run(["g++", "-shared", "-o", lib] + objs + ["-lpthread"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference link failed:\n" + r.stderr[-4000:])
    with open(stamp, "w") as f:
        f.write(key)
    if not quiet:
        print("built", lib)
    return lib


def build_sampler(quiet=True):
    """Compile the reference sampler driver (host code, nvcc) against the checkout's headers;
    returns the .so path or None without a checkout."""
    if not have_checkout():
        return None
    lib = os.path.join(OUT, "libifrit_ref_sampler.so")
    src = os.path.join(HERE, "ref_sampler.cu")
    if os.path.exists(lib) and os.path.getmtime(lib) >= os.path.getmtime(src):
        return lib
    os.makedirs(OUT, exist_ok=True)
    cmd = [NVCC, "-std=c++20", "-O2", "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off", "-w",
           "-DIFRIT_FEATURE_CUDA", "-DIFRIT_DLL", "-I" + os.path.join(REF_ROOT, "include"), src, "-o", lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference sampler build failed:\n" + r.stderr[-4000:])
    if not quiet:
        print("built", lib)
    return lib


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what in ("stage", "all"):
        print(stage() if have_checkout() else "no checkout (IFRIT_REFERENCE_ROOT)")
    if what in ("renderer", "all"):
        print(build(quiet=False))
    if what in ("scalar", "all"):
        print(build(simd=False, quiet=False))
    if what in ("sampler", "all"):
        print(build_sampler(quiet=False))
