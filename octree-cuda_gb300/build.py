"""Build recipe of the native libraries (no cmake): nvcc for the sm_103a
kernels, the host C++ compiler for the session/orchestration code.

Outputs (in this directory, git-ignored):
  libOctreeApi.so  -- the C-ABI LOD octree builder (the product)
  libocsynth.so    -- seeded synthetic clouds + the CLI's bounding box helper
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["k_chunking.cu", "k_subsample.cu", "noalloc.cu"]
CPP_SOURCES = ["builder.cpp", "export.cpp", "octree_api.cpp", "serve.cpp", "wave.cpp"]
HEADERS = ["device_common.cuh", "kernels.h", "builder.h", "wave.h"]

LIB = os.path.join(HERE, "libOctreeApi.so")
SYNTH_LIB = os.path.join(HERE, "libocsynth.so")


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


EXTRA_NVCC = os.environ.get("OC_EXTRA_NVCC", "").split()


def _compile(src, verbose_ptxas=False):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    deps = [path] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "octreeApi.h")]
    if _newer(obj, deps) and not verbose_ptxas:
        return obj, ""
    if src.endswith(".cu"):
        cmd = [NVCC, *ARCH, *EXTRA_NVCC, "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-fvisibility=hidden", "-c", path, "-o", obj]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off",
               "-I" + os.path.join(CUDA_HOME, "include"), "-c", path, "-o", obj]
    out = _run(cmd)
    return obj, out


def build(force=False, verbose_ptxas=False):
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    sources = CU_SOURCES + CPP_SOURCES
    with cf.ThreadPoolExecutor(max_workers=len(sources)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), sources))
    objs = [r[0] for r in results]
    logs = "".join(r[1] for r in results)
    if not _newer(LIB, objs) or force:
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fPIC"])
    synth_src = os.path.join(CSRC, "synthetic.cpp")
    if force or not _newer(SYNTH_LIB, [synth_src]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", synth_src, "-o", SYNTH_LIB])
    return logs


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    for f in (LIB, SYNTH_LIB):
        if os.path.exists(f):
            os.remove(f)


if __name__ == "__main__":
    log = build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv)
    if log.strip():
        print(log)
    print(LIB)
