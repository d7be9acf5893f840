"""Build libcfft_gb300.so in-tree for sm_103a (nvcc + g++, no cmake).

    python concrete-fft_gb300/build.py [--force] [-j N]

Each translation unit is compiled in parallel into concrete-fft_gb300/_build/
and linked into concrete-fft_gb300/lib/libcfft_gb300.so.  Device code is
compiled with --fmad=false and host code with -ffp-contract=off: the library's
results are defined as the exact IEEE operation sequence of the reference, so
no multiply-add may be fused that the reference keeps separate.
"""
import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib", "libcfft_gb300.so")

CUDA_SOURCES = ["c64.cu", "product_u64.cu", "f128.cu", "runtime.cu", "batch.cu", "product_engine.cu", "server.cu", "queue.cu", "kinst_c64_e0.cu", "kinst_c64_emu.cu", "kinst_prod_e0.cu", "kinst_prod_emu.cu", "kinst_split_01.cu", "kinst_split_23.cu", "kinst_split_45.cu", "kinst_split_67.cu", "kinst_split_prod_01.cu", "kinst_split_prod_23.cu", "kinst_split_prod_45.cu", "kinst_split_prod_67.cu"]
CXX_SOURCES = ["twiddles.cpp", "tune_cache.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _deps(src):
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    return [src] + headers + [os.path.join(ROOT, "include", "cfft.h")]


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, force):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if not force and not _stale(obj, _deps(path)):
        return obj, None
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "--fmad=false", "-std=c++17", "-Xcompiler",
               "-fPIC,-ffp-contract=off", "-Xptxas", "-v", "-c", path, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
               "-fno-fast-math", "-I", os.path.join(cuda_home(), "include"), "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    with open(obj + ".log", "w") as f:
        f.write(r.stdout + r.stderr)
    return obj, r.stderr


def build(force=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    sources = CUDA_SOURCES + CXX_SOURCES
    with ThreadPoolExecutor(max_workers=jobs or len(sources)) as ex:
        results = list(ex.map(lambda s: _compile(s, force), sources))
    objs = [o for o, _ in results]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    return LIB


def build_oracle(force=False):
    odir = os.path.join(ROOT, "oracle")
    cmd = ["make", "-s", "-C", odir] + (["-B"] if force else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s\n%s" % (r.stdout, r.stderr))
    return os.path.join(odir, "liboracle.so")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    args = ap.parse_args()
    print(build(args.force, args.j))
