"""Builds libsesnt.so (the GB300 time step behind include/sesnt.h) in place.

Host set-up code is compiled with g++ and -ffp-contract=off so its float32
arithmetic matches the reference's rounding on x86-64 and aarch64 alike; the
CUDA translation units are compiled for sm_103a only. Translation units are
compiled in parallel.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsesnt.so")
CLI = os.path.join(HERE, "ses3d-nt-gpu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def build(verbose=False, extra_nvcc=(), out_dir=None):
    """Compile every translation unit and link libsesnt.so. Returns its path.
    out_dir: build a separate library there (objects and libsesnt.so, no
    CLI), e.g. the bounds-check build with extra_nvcc=["-DSESNT_BOUNDS_CHECK"]."""
    build_dir = os.path.join(out_dir, "_build") if out_dir else BUILD
    lib = os.path.join(out_dir, "libsesnt.so") if out_dir else LIB
    os.makedirs(build_dir, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = sources()
    jobs = []
    for f in cu:
        obj = os.path.join(build_dir, f + ".o")
        jobs.append(([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-I", INCLUDE,
                      "-Xcompiler", "-fPIC,-ffp-contract=off", *extra_nvcc,
                      "-c", os.path.join(CSRC, f), "-o", obj], obj))
    for f in cpp:
        obj = os.path.join(build_dir, f + ".o")
        jobs.append((["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                      "-I", INCLUDE, "-I", "/usr/local/cuda/include",
                      "-c", os.path.join(CSRC, f), "-o", obj], obj))
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        outs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [o for _, o in jobs]
    _run([nvcc, *ARCH, "-shared", "-o", lib + ".tmp", *objs, "-Xcompiler", "-fPIC"])
    os.replace(lib + ".tmp", lib)
    if out_dir:
        return lib
    # command-line driver linked against the library (found next to it)
    _run(["g++", "-O2", "-std=c++17", "-o", CLI + ".tmp", os.path.join(HERE, "cli", "ses3d-nt-gpu.cpp"),
          "-L" + HERE, "-lsesnt", "-Wl,-rpath,$ORIGIN"])
    os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
