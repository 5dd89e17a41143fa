"""Build libbfgb300.so (CUDA for sm_103a + the C ABI) in-tree.

    python boostfractor.jl_gb300/build.py [--force]

Translation units compile in parallel with one -gencode; the host side is
compiled with -ffp-contract=off so host geometry rounds identically on
x86-64 and aarch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libbfgb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["bf_device.cu", "bf_api.cu", "bf_transformer.cu", "bf_noalloc.cu", "bf_tcgemm.cu", "bf_server.cpp", "bf_modes.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I", CSRC, "-I", INCLUDE, "--expt-relaxed-constexpr"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + \
        [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def build(force=False, verbose=False):
    os.makedirs(OBJDIR, exist_ok=True)
    deps = _deps()
    if not force and not _newer(LIB, deps + [os.path.abspath(__file__)]):
        return LIB
    nv = nvcc()
    jobs = []
    for src in SOURCES:
        obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
        cmd = [nv] + _flags() + ["-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, obj))

    def run(job):
        cmd, obj = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
