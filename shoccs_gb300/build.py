"""Build the in-tree CUDA library libshoccs_gb300.so for sm_103a and the shoccs command line
over it.

Compiles the device kernels with nvcc and the host setup / C ABI with g++, in parallel,
into shoccs_gb300/_build/.  Host code is built with -ffp-contract=off so the setup
arithmetic (ray casts, closure coefficients) rounds identically on x86-64 and aarch64.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
APP = os.path.join(HERE, "app")
INCLUDE = os.path.join(HERE, "..", "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libshoccs_gb300.so")
CLI = os.path.join(BUILD, "shoccs")  # the command line (app/shoccs.cpp) over the library
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = ["host/problem.cpp", "capi.cpp"]
CUDA_SOURCES = ["kernels.cu"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _deps():
    out = []
    for root, _, files in os.walk(CSRC):
        out += [os.path.join(root, f) for f in files if f.endswith((".cpp", ".cu", ".hpp", ".cuh", ".h"))]
    out.append(os.path.join(HERE, "..", "include", "shoccs_gpu.h"))
    return out


def _build_cli(force):
    deps = [os.path.join(APP, f) for f in os.listdir(APP) if f.endswith((".cpp", ".hpp"))]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)] + [LIB]
    if not force and _newer(CLI, deps + [os.path.abspath(__file__)]):
        return
    _run(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-I" + INCLUDE, "-I" + APP,
          "-I" + os.path.join(CUDA_HOME, "include"), os.path.join(APP, "shoccs.cpp"), "-o", CLI,
          "-L" + BUILD, "-lshoccs_gb300", "-L" + os.path.join(CUDA_HOME, "lib64"), "-lcudart",
          "-Wl,-rpath,$ORIGIN"])


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    if not force and _newer(LIB, deps + [os.path.abspath(__file__)]):
        _build_cli(force)
        return LIB
    inc = ["-I" + CSRC, "-I" + os.path.join(CUDA_HOME, "include")]
    jobs = []
    objs = []
    for src in HOST_SOURCES:
        obj = os.path.join(BUILD, os.path.basename(src).replace(".cpp", ".o"))
        objs.append(obj)
        jobs.append(["g++", "-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                     "-Wno-unused-variable"] + inc + ["-c", os.path.join(CSRC, src), "-o", obj])
    for src in CUDA_SOURCES:
        obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".cu.o"))
        objs.append(obj)
        jobs.append([NVCC] + ARCH + ["-std=c++20", "-O3", "-lineinfo", "-Xptxas", "-v",
                     "-Xcompiler", "-fPIC,-ffp-contract=off"] + inc + ["-c", os.path.join(CSRC, src), "-o", obj])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for l in logs:
            sys.stderr.write(l)
    _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    _build_cli(True)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
