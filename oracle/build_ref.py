"""Staging and compile recipe for the reference (PotreeConverterGPU) -- TEST
INFRASTRUCTURE ONLY.

  stage()    copies the reference's Potree reader tools/potree_to_ply.py
             (standard-library Python) from the reference checkout
             (OC_REFERENCE_DIR, default /root/reference) into the git-ignored
             oracle/_ref/tools; the GPU tests run it on this library's export.
             It runs where the checkout exists; the staged copy travels with the
             working tree to machines where it does not.  Never committed.
  compile()  compiles the reference's 13 OctreeApi/OctreeLibrary translation
             units, unmodified and where they lie in the checkout, for sm_103a
             into oracle/_ref/obj and archives them as
             oracle/_ref/libOctreeApiRef.a.  oracle/ref_shim.h is
             force-included into each (an 8-byte atomicAdd overload and a clock
             alias; see that file).  Flags follow the reference's CMake build
             (separable compilation, header-only spdlog) with release
             optimisation.  Compile only: the reference pipeline is not run on a
             GPU here, because it accessed memory outside its buffers on every
             cloud it was given (its subsampling reads node fields that nothing
             initialises).

    python oracle/build_ref.py            # stage the reader
    python oracle/build_ref.py --compile  # compile the reference library
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("OC_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")
SRC = REF_DIR
OBJ = os.path.join(OUT, "obj")
ARCHIVE = os.path.join(OUT, "libOctreeApiRef.a")
READER = os.path.join(OUT, "tools", "potree_to_ply.py")
SHIM = os.path.join(HERE, "ref_shim.h")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

LIB = "OctreeApi/OctreeLibrary"
INCLUDE_DIRS = [
    "External", "External/nlohmann", "External/spdlog/include",
    LIB + "/include", LIB + "/src/include", LIB + "/src/kernel", LIB + "/src/misc",
    LIB + "/src/octree_exporter", LIB + "/src/data",
    "OctreeApi/include", "OctreeApi/src", "src",
]


def stage():
    """Copy the reference's Potree reader into oracle/_ref/tools.  Returns
    True when a staged copy exists afterwards."""
    src = os.path.join(REF_DIR, "tools", "potree_to_ply.py")
    if os.path.exists(src) and not _newer(READER, [src]):
        os.makedirs(os.path.dirname(READER), exist_ok=True)
        shutil.copy2(src, READER)
    return os.path.exists(READER)


def _library_sources():
    srcs = []
    for root, _, files in os.walk(os.path.join(SRC, LIB, "src")):
        srcs += [os.path.join(root, f) for f in files if f.endswith(".cu")]
    srcs += [os.path.join(SRC, "OctreeApi/src", f) for f in ("octreeApi.cpp", "session.cpp")]
    return sorted(srcs)


def _headers():
    hs = [SHIM]
    for root, _, files in os.walk(os.path.join(SRC, LIB)):
        hs += [os.path.join(root, f) for f in files if f.endswith((".cuh", ".h"))]
    return hs


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed: %s\n%s%s" % (" ".join(cmd), r.stdout[-4000:], r.stderr[-4000:]))


def _compile(src, headers):
    name = os.path.relpath(src, SRC).replace("/", "_") + ".o"   # objects only under oracle/_ref
    obj = os.path.join(OBJ, name)
    if _newer(obj, [src] + headers):
        return obj
    inc = ["-I" + os.path.join(SRC, d) for d in INCLUDE_DIRS]
    cmd = [NVCC, *ARCH, "-std=c++17", "-O3", "-DNDEBUG", "-rdc=true", "-x", "cu", "-w",
           "-include", SHIM, *inc, "-c", src, "-o", obj]
    _run(cmd)
    return obj


def compile(jobs=None):
    """Compile the reference library from the checkout.  Returns the archive
    path, or None when the checkout or nvcc is absent."""
    if not os.path.isdir(os.path.join(SRC, LIB)) or not os.path.exists(NVCC):
        return None
    os.makedirs(OBJ, exist_ok=True)
    headers = _headers()
    srcs = _library_sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda src: _compile(src, headers), srcs))
    if not _newer(ARCHIVE, objs):
        if os.path.exists(ARCHIVE):
            os.remove(ARCHIVE)
        _run(["ar", "rcs", ARCHIVE, *objs])
    return ARCHIVE


def reader():
    """Path of the staged Potree reader, or None."""
    return READER if os.path.exists(READER) else None


if __name__ == "__main__":
    if "--compile" in sys.argv:
        path = compile()
        print(path if path else "reference checkout unavailable: nothing compiled")
    else:
        print("staged" if stage() else "reference checkout unavailable")
