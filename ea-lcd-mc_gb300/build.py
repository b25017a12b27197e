"""Build libeagb.so in-tree for sm_103a (nvcc, no CMake).

    python ea-lcd-mc_gb300/build.py [--clean]

Translation units compile in parallel; the library lands next to this file
as libeagb.so together with the ea_gb command-line driver.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libeagb.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-Xcompiler", "-fPIC"]
SOURCES = ["kernels.cu", "batch.cu", "api.cu", "host.cpp", "noalloc.cu", "serve.cpp", "sp.cu", "sp_resident.cu", "sp_analysis.cu", "sp_host.cpp", "probe.cu"]


def _compile(src):
    out = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".hpp", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "eagb.h"))
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
        return out
    cmd = [NVCC] + ARCH + COMMON + ["-lineinfo", "-Xptxas", "-v", "-c", path, "-o", out]
    if src.endswith(".cpp"):
        cmd = [NVCC] + COMMON + ["-x", "c++", "-c", path, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    with open(out + ".log", "w") as f:
        f.write(r.stdout + r.stderr)
    return out


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcurand", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stderr))
    exe = os.path.join(HERE, "ea_gb")
    src = os.path.join(CSRC, "ea_gb.cpp")
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(LIB), os.path.getmtime(src)):
        cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), src, "-o", exe,
               "-L" + HERE, "-leagb", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver build failed: %s\n%s" % (" ".join(cmd), r.stderr))
    if verbose:
        for o in objs:
            if os.path.exists(o + ".log"):
                print(open(o + ".log").read())
    return LIB


if __name__ == "__main__":
    if "--clean" in sys.argv:
        shutil.rmtree(BUILD, ignore_errors=True)
        if os.path.exists(LIB):
            os.remove(LIB)
    print(build(verbose="-v" in sys.argv))
