"""Recipe that builds the reference's own CUDA pipeline -- TEST INFRASTRUCTURE ONLY.

The reference (PotreeConverterGPU: OctreeApi + OctreeLibrary) is the parity
oracle on the GPU and the timed reference arm.  It is compiled from its own
sources, unmodified, for sm_103a; nothing of it is committed:

  stage()  copies the files the build needs (the OctreeApi library, the CLI's
           bounding-box header, the header-only spdlog and nlohmann json it
           includes, and the Potree reader tools/potree_to_ply.py) from the
           reference checkout into the git-ignored oracle/_ref/src.  It runs
           where the checkout exists (OC_REFERENCE_DIR, default
           /root/reference); the staged copy travels to the GPU machine with
           the working tree, where the checkout does not exist.
  build()  compiles the staged sources with nvcc into oracle/_ref/ref_runner.
           The 13 translation units of the library are compiled exactly as
           they are; oracle/ref_shim.h is force-included into each of them
           (an 8-byte atomicAdd overload and a clock alias; see that file).
           oracle/ref_runner.cpp is this project's driver of the reference's
           C API.  Objects are rebuilt only when a source is newer.

Flags follow the reference's CMake build (OctreeApi/OctreeLibrary/
CMakeLists.txt: separable compilation, header-only spdlog) with release
optimisation: -O3 -DNDEBUG.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("OC_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
OBJ = os.path.join(OUT, "obj")
RUNNER = os.path.join(OUT, "ref_runner")
READER = os.path.join(SRC, "tools", "potree_to_ply.py")
SHIM = os.path.join(HERE, "ref_shim.h")
DRIVER = os.path.join(HERE, "ref_runner.cpp")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# Directories and files of the reference checkout that the build reads.
STAGE_TREES = [
    "OctreeApi/include",
    "OctreeApi/src",
    "OctreeApi/OctreeLibrary/include",
    "OctreeApi/OctreeLibrary/src",
    "External/spdlog/include",
    "External/nlohmann",
]
STAGE_FILES = ["src/boundingbox.h", "tools/potree_to_ply.py"]

LIB = "OctreeApi/OctreeLibrary"
INCLUDE_DIRS = [
    "External", "External/nlohmann", "External/spdlog/include",
    LIB + "/include", LIB + "/src/include", LIB + "/src/kernel", LIB + "/src/misc",
    LIB + "/src/octree_exporter", LIB + "/src/data",
    "OctreeApi/include", "OctreeApi/src", "src",
]


def staged():
    """True when oracle/_ref/src holds a staged copy of the reference."""
    return os.path.exists(os.path.join(SRC, "STAGED"))


def stage(force=False):
    """Copy the reference files the build needs into oracle/_ref/src.

    Returns True when a staged copy exists afterwards."""
    if not os.path.isdir(REF_DIR):
        return staged()
    if staged() and not force:
        return True
    tmp = SRC + ".tmp"
    shutil.rmtree(tmp, ignore_errors=True)
    for tree in STAGE_TREES:
        shutil.copytree(os.path.join(REF_DIR, tree), os.path.join(tmp, tree))
    for f in STAGE_FILES:
        os.makedirs(os.path.dirname(os.path.join(tmp, f)), exist_ok=True)
        shutil.copy2(os.path.join(REF_DIR, f), os.path.join(tmp, f))
    with open(os.path.join(tmp, "STAGED"), "w") as fh:
        fh.write("copied from %s; never committed\n" % REF_DIR)
    shutil.rmtree(SRC, ignore_errors=True)
    os.rename(tmp, SRC)
    return True


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


def _compile(src, headers, shim=True):
    name = os.path.relpath(src, SRC).replace("/", "_") + ".o"
    obj = os.path.join(OBJ, name)
    if _newer(obj, [src] + headers):
        return obj
    inc = ["-I" + os.path.join(SRC, d) for d in INCLUDE_DIRS]
    cmd = [NVCC, *ARCH, "-std=c++17", "-O3", "-DNDEBUG", "-rdc=true", "-x", "cu", "-w",
           *(["-include", SHIM] if shim else []), *inc, "-c", src, "-o", obj]
    _run(cmd)
    return obj


def build(jobs=None):
    """Compile the staged reference and the runner.  Returns the runner path,
    or None when no staged copy or no nvcc is present."""
    if not stage() or not os.path.exists(NVCC):
        return None
    os.makedirs(OBJ, exist_ok=True)
    headers = _headers()
    srcs = _library_sources()
    jobs = jobs or min(len(srcs) + 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile, s, headers) for s in srcs]
        futs.append(ex.submit(_compile, DRIVER, headers, False))
        objs = [f.result() for f in futs]
    if not _newer(RUNNER, objs):
        _run([NVCC, *ARCH, "-rdc=true", "-o", RUNNER, *objs])
    return RUNNER


def runner():
    """Path of the built runner, or None."""
    return RUNNER if os.path.exists(RUNNER) else None


if __name__ == "__main__":
    if "--stage" in sys.argv:
        print("staged" if stage(force=True) else "reference sources unavailable")
    else:
        path = build()
        print(path if path else "reference sources unavailable: nothing built")
