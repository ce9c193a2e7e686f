"""Builds the GB300 shared library ``mini_mdft_gb300/lib/libmdft_gb300.so``.

Every translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel, then linked with
the static CUDA runtime.  The library exports exactly the C ABI declared in
``include/mdft_gb300.h``; nothing in it depends on PyTorch.
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libmdft_gb300.so")
HEADER = os.path.join(ROOT, "include", "mdft_gb300.h")

CU_SOURCES = ["capi.cu", "angular.cu", "angular_tc.cu", "angular_fast_f64.cu", "angular_fast_f32.cu", "angular_fast_df.cu", "fft_f64.cu", "fft_f32.cu", "fft_df.cu", "oz_f64.cu", "oz_f32.cu", "oz_df.cu", "oz_r2_f32.cu", "oz_r2_df.cu", "energy.cu", "server.cu", "solver.cu"]
CPP_SOURCES = ["host_setup.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    return hdrs + [HEADER]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + _deps())


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _host_stamp_ok():
    """Objects built on another host architecture are never reused."""
    stamp = os.path.join(OBJ, "HOST")
    ok = os.path.exists(stamp) and open(stamp).read().strip() == platform.machine()
    return ok, stamp


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    ok, stamp = _host_stamp_ok()
    if not ok:
        force = True
    jobs = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                   "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
            if ptxas_v:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for f in CPP_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                         "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_compile, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or not os.path.exists(LIB):
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", LIB + ".tmp", *objs]
        _compile(cmd)
        os.replace(LIB + ".tmp", LIB)
        with open(stamp, "w") as f:
            f.write(platform.machine())
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv))
