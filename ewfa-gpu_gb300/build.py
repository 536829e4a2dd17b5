"""Build recipe of libwfe (sm_103a) and its tools, in-tree.

    python ewfa-gpu_gb300/build.py   # lib/libwfe.so, lib/libwfe_gen.so, lib/libwfe_intpeak.so,
                                     # bin/wfe.aligner, bin/wfe.gen

Outputs go to ewfa-gpu_gb300/_build (objects), lib/ and bin/.  Translation
units compile in parallel; a unit is rebuilt only when it or a header it may
include is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
BIN = os.path.join(PKG, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# relocatable device code: the tier kernels launch their successors on the
# device (tail launches), which needs the device runtime (cudadevrt)
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-rdc=true", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              f"-I{INC}", f"-I{CSRC}"] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wextra", f"-I{INC}", f"-I{CSRC}"]
CC_FLAGS = ["-O2", "-std=c11", "-fPIC", "-Wall", "-Wextra", "-ffp-contract=off", f"-I{INC}", f"-I{CSRC}"]

LIB_CU = ["wfe_kernels.cu", "wfe_api.cu", "wfe_noalloc.cu", "wfe_server.cu"]
LIB_CXX = ["wfe_host.cpp", "seqfile.cpp"]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _headers() -> list[str]:
    hs = [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build(verbose: bool = False) -> dict:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for f in LIB_CU:
        src, obj = os.path.join(CSRC, f), os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj])
    for f in LIB_CXX:
        src, obj = os.path.join(CSRC, f), os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    gen_src = os.path.join(CSRC, "wfe_gen.c")
    gen_obj = os.path.join(OBJ, "wfe_gen.c.o")
    if _stale(gen_obj, [gen_src] + hdrs):
        jobs.append(["gcc"] + CC_FLAGS + ["-c", gen_src, "-o", gen_obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs)))) as ex:
        list(ex.map(_run, jobs))

    libwfe = os.path.join(LIB, "libwfe.so")
    if _stale(libwfe, objs):
        _run([nvcc] + ARCH + ["-shared", "-rdc=true", "-o", libwfe] + objs + ["-lcudadevrt", "-lpthread"])
    libgen = os.path.join(LIB, "libwfe_gen.so")
    if _stale(libgen, [gen_obj]):
        _run(["gcc", "-shared", "-o", libgen, gen_obj, "-lm", "-lpthread"])
    # the integer-issue peak probe that the benchmark's integer roofline divides by
    peak_src = os.path.join(CSRC, "int_peak.cu")
    libpeak = os.path.join(LIB, "libwfe_intpeak.so")
    if _stale(libpeak, [peak_src]):
        _run([nvcc, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-shared"] + ARCH +
             [peak_src, "-o", libpeak])

    # command-line tools, linked against the shared library
    cuda_lib = os.path.join(_cuda_home(), "lib64")
    tools = {
        "wfe.aligner": (["aligner.cpp"], ["-lwfe"]),
        "wfe.gen": (["gen_main.c"], ["-lwfe_gen"]),
    }
    for name, (srcs, libs) in tools.items():
        paths = [os.path.join(CSRC, s) for s in srcs]
        if not all(os.path.exists(p) for p in paths):
            continue
        out = os.path.join(BIN, name)
        if _stale(out, paths + hdrs + [libwfe, libgen]):
            comp = "g++" if any(p.endswith(".cpp") for p in paths) else "gcc"
            flags = CXX_FLAGS if comp == "g++" else CC_FLAGS
            _run([comp] + [f for f in flags if f != "-fPIC"] + paths + ["-o", out, f"-L{LIB}"] + libs +
                 [f"-Wl,-rpath,$ORIGIN/../lib", f"-L{cuda_lib}", "-lpthread", "-lm"])
    res = {"libwfe": libwfe, "libwfe_gen": libgen, "bin": BIN}
    if verbose:
        print(res)
    return res


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
