"""Build libbrick_gb300.so in-tree with nvcc for sm_103a.

Each translation unit under csrc/ compiles in parallel into _build/, then nvcc links
the shared library into bricklib_gb300/lib/.  Only the translation units whose
source or headers changed are recompiled.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libbrick_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
          "--expt-relaxed-constexpr"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps_mtime() -> float:
    hdrs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hdrs), default=0.0)


def _extra_flags() -> list:
    """BK_NVCC_FLAGS: extra nvcc flags for experiments with the kernels' build-time switches
    (e.g. -DBK_CS_SWZ=0); a change of them rebuilds every translation unit."""
    return os.environ.get("BK_NVCC_FLAGS", "").split()


def _flags_changed() -> bool:
    stamp = os.path.join(BUILD, "flags.txt")
    want = " ".join(_extra_flags())
    have = open(stamp).read() if os.path.exists(stamp) else ""
    if have != want:
        with open(stamp, "w") as f:
            f.write(want)
        return True
    return False


def _compile(src: str, verbose: bool, force: bool = False) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _deps_mtime()):
        return obj
    cmd = [nvcc()] + ARCH + CFLAGS + _extra_flags() + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    force = _flags_changed()
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, force), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def build_cpp_driver(verbose: bool = False) -> str:
    """The C++ drop-in driver of tests/cpp/single_gb300.cpp, linked against the library."""
    src = os.path.join(ROOT, "tests", "cpp", "single_gb300.cpp")
    exe = os.path.join(LIBDIR, "single_gb300")
    deps = [src, LIB] + glob.glob(os.path.join(INCLUDE, "*.h"))
    if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(d) for d in deps):
        return exe
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
    cmd = ["g++", "-O2", "-fopenmp", "-std=c++17", "-I", INCLUDE, "-I", cuda_inc, src, "-o", exe,
           "-L", LIBDIR, "-lbrick_gb300", "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed on {src}:\n{r.stdout}\n{r.stderr}")
    return exe


def build_lowered_program(src: str, exe: str, verbose: bool = False) -> str:
    """A C++ brick program with brick("x.py", ...) statements: lowered by
    bricklib_gb300.dsl.vecscatter (as the reference's build runs its code generator first),
    then compiled and linked against the library."""
    from .dsl import vecscatter
    lib = build()
    with open(src) as f:
        text, report = vecscatter.lower_source(f.read(), os.path.abspath(src))
    missed = [r for r in report if not r["lowered"]]
    if missed:
        raise RuntimeError(f"{src}: brick(...) statements not lowered: {missed}")
    lowered = exe + ".lowered.cpp"
    with open(lowered, "w") as f:
        f.write(text)
    cuda = os.path.dirname(os.path.dirname(nvcc()))
    cmd = ["g++", "-O2", "-fopenmp", "-std=c++17", "-I", INCLUDE, "-I", os.path.join(cuda, "include"),
           "-I", os.path.dirname(os.path.abspath(src)), lowered, "-o", exe, "-L", os.path.dirname(lib),
           "-lbrick_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.dirname(lib)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed on the lowered {src}:\n{r.stdout}\n{r.stderr}")
    return exe


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
    print(build_cpp_driver(verbose="-v" in sys.argv))
