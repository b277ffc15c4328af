"""Build the path_gb300 shared library in-tree.

Compiles path_gb300/csrc (CUDA kernels for sm_103a with nvcc, host C++ with
g++) into path_gb300/_lib/libpath_gb300.so.  The translation units are
compiled in parallel.  Floating-point contraction is disabled everywhere
(--fmad=false for device code, -ffp-contract=off for host code) because the
kernels must reproduce the host-side arithmetic bit for bit.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libpath_gb300.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["render.cu", "sobol.cu", "noalloc.cu", "wavefront.cu", "cache.cu",
              "nrc_paths.cu", "gpu_build.cu"]
CPP_SOURCES = ["capi.cpp", "renderer.cpp", "batch.cpp", "cache_host.cpp", "scene.cpp",
               "scene_load.cpp", "sbvh.cpp", "wide.cpp", "settings.cpp"]

INCLUDES = ["-I" + CSRC, "-I" + os.path.join(ROOT, "include"),
            "-I" + os.path.join(CUDA_HOME, "include")]

# How the integrator draws its Sobol numbers: "table" reads the [spp][dims]
# table built once per render (the reference's scheme), "direct" forms each
# value from the direction vectors XOR-ed in a register.  Both give the same
# values bit for bit; the choice is a build option (PATH_GB300_SOBOL_DRAW).
SOBOL_DRAW = os.environ.get("PATH_GB300_SOBOL_DRAW", "table")
STAMP = os.path.join(OUT_DIR, "build_options.txt")


def _sources_newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _all_deps():
    deps = []
    for d in (CSRC, os.path.join(ROOT, "include")):
        for name in os.listdir(d):
            if name.endswith((".h", ".cuh", ".cu", ".cpp")):
                deps.append(os.path.join(d, name))
    return deps


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    return proc.stdout


def _options():
    if SOBOL_DRAW not in ("table", "direct"):
        raise RuntimeError("PATH_GB300_SOBOL_DRAW must be 'table' or 'direct'")
    return f"sobol_draw={SOBOL_DRAW}"


def build(force=False, verbose=False, ptxas_info=False):
    """Compile the library if any source is newer than it (or the build
    options changed); return its path."""
    deps = _all_deps()
    try:
        with open(STAMP) as f:
            same_options = f.read() == _options()
    except OSError:
        same_options = False
    if not force and same_options and not _sources_newer(LIB, deps):
        return LIB
    if shutil.which(NVCC) is None and not os.path.exists(NVCC):
        raise RuntimeError("nvcc not found at " + NVCC)
    obj_dir = os.path.join(OUT_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(obj_dir, src + ".o")
        cmd = [NVCC] + ARCH + ["-lineinfo", "-O3", "--fmad=false", "-std=c++17",
                               "-Xcompiler", "-fPIC,-ffp-contract=off",
                               f"-DPG_SOBOL_DIRECT={1 if SOBOL_DRAW == 'direct' else 0}",
                               "-c", os.path.join(CSRC, src), "-o", obj] + INCLUDES
        if ptxas_info:
            cmd += ["-Xptxas", "-v"]
        jobs.append((cmd, obj))
    for src in CPP_SOURCES:
        obj = os.path.join(obj_dir, src + ".o")
        cmd = ["g++", "-O3", "-std=gnu++17", "-fPIC", "-ffp-contract=off", "-fopenmp",
               "-Wall", "-c", os.path.join(CSRC, src), "-o", obj] + INCLUDES
        jobs.append((cmd, obj))
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        outs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose or ptxas_info:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp"
    link = [NVCC] + ARCH + ["-shared", "-o", tmp] + [o for _, o in jobs] + [
        "-L" + os.path.join(CUDA_HOME, "lib64"), "-lcurand", "-lgomp",
        "-Xlinker", "-rpath," + os.path.join(CUDA_HOME, "lib64")]
    _run(link)
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(_options())
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
