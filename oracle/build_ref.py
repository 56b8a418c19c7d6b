"""Build recipe for the reference CPU tile rasterizer (test infrastructure only).

Compiles the reference's own CPU renderer sources where they lie under the read-only
reference checkout, together with ``oracle/ref_driver.cpp``, into
``oracle/_ref/libifrit_ref.so``.  Nothing from the reference is copied into the
repository: the two header overlays the build needs are generated into the git-ignored
``oracle/_ref/overlay/`` at build time:

* ``ifrit/core/typing/Util.h``: the dead ``#ifdef __PRETTY_FUNCTION__`` branch ending in
  ``static_assert(false)`` (include/ifrit/core/typing/Util.h:113-124) is rejected by
  GCC 13; the overlay keeps only the ``__PRETTY_FUNCTION__`` return.
* ``ifrit/softgraphics/engine/tileraster/TileRasterContext.h``: ``numThreads`` (a
  compile-time constant, 16 in the reference, TileRasterContext.h:52) is set to the
  host's core count minus one, because the reference's spin barriers degrade sharply
  when oversubscribed.

The reference's CPU path uses x86 AVX2 intrinsics unconditionally in three places
(Image.h:110-113, TileRasterWorker.cpp:1689-1690, 1938-1939), so this recipe only
builds on x86_64; on other hosts ``build()`` reports the reference as unavailable.
"""
import os
import platform
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_ROOT = os.environ.get("IFRIT_REFERENCE_ROOT", "/root/reference")

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

FLAGS = ["-std=c++20", "-O2", "-fPIC", "-mavx2", "-mfma", "-DIFRIT_FEATURE_SIMD=1",
         "-DIFRIT_FEATURE_SIMD_AVX256=1", "-DIFRIT_DLL", "-DIFRIT_API_EXPORT", "-w"]


def available():
    return platform.machine() in ("x86_64", "AMD64") and os.path.isdir(REF_ROOT)


def _write_overlay(num_threads):
    inc = os.path.join(REF_ROOT, "include")
    util_src = open(os.path.join(inc, "ifrit/core/typing/Util.h")).read()
    pat = re.compile(r"#ifdef __PRETTY_FUNCTION__\s*return __PRETTY_FUNCTION__;\s*#else\s*"
                     r"static_assert\(false, \"Unsupported compiler\"\);\s*#endif")
    util_new, n = pat.subn("return __PRETTY_FUNCTION__;", util_src)
    if n != 1:
        raise RuntimeError("Util.h overlay pattern not found")
    ctx_src = open(os.path.join(inc, "ifrit/softgraphics/engine/tileraster/TileRasterContext.h")).read()
    ctx_new, n = re.subn(r"(IF_CONSTEXPR static int numThreads\s*=\s*)16;", r"\g<1>%d;" % num_threads, ctx_src)
    if n != 1:
        raise RuntimeError("TileRasterContext.h overlay pattern not found")
    for rel, text in (("ifrit/core/typing/Util.h", util_new),
                      ("ifrit/softgraphics/engine/tileraster/TileRasterContext.h", ctx_new)):
        path = os.path.join(OUT, "overlay", rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            f.write(text)


def build(num_threads=None, quiet=True):
    """Compile the reference renderer + driver; returns the .so path or None."""
    if not available():
        return None
    if num_threads is None:
        num_threads = max(1, (os.cpu_count() or 2) - 1)
    lib = os.path.join(OUT, "libifrit_ref.so")
    stamp = os.path.join(OUT, "threads.txt")
    driver = os.path.join(HERE, "ref_driver.cpp")
    if (os.path.exists(lib) and os.path.exists(stamp) and open(stamp).read().strip() == str(num_threads)
            and os.path.getmtime(lib) >= os.path.getmtime(driver)):
        return lib
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    _write_overlay(num_threads)
    incs = ["-I" + os.path.join(OUT, "overlay"), "-I" + os.path.join(REF_ROOT, "include")]
    jobs = []
    for rel in SOURCES + [driver]:
        src = rel if os.path.isabs(rel) else os.path.join(REF_ROOT, rel)
        obj = os.path.join(OUT, "obj", os.path.basename(src) + ".o")
        jobs.append((["g++"] + FLAGS + incs + ["-c", src, "-o", obj], obj))

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
        f.write(str(num_threads))
    if not quiet:
        print("built", lib)
    return lib


if __name__ == "__main__":
    n = int(sys.argv[1]) if len(sys.argv) > 1 else None
    print(build(n, quiet=False))
