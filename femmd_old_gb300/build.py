"""Build of libfemmd.so, the CUDA library behind the femmd2D timestep.

nvcc, sm_103a only, in-tree: objects go to femmd_old_gb300/_build/, the
library to femmd_old_gb300/libfemmd.so.  Translation units compile in
parallel.  Device code is compiled with -fmad=false and host code with
-ffp-contract=off so that no multiply-add is contracted: the kernels and the
host setup reproduce the reference's single-precision arithmetic bit for bit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
SRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libfemmd.so")
SOURCES = ["k_nn.cu", "k_force.cu", "k_fast.cu", "k_batch.cu", "k_adjoint.cu", "k_props.cu", "femmd_api.cu", "k_bin_noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                "-I" + os.path.join(ROOT, "include"), "-I" + SRC]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "femmd.h"))
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(SRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + FLAGS + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose:
            sys.stdout.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs)
    return LIB


FRONTEND = os.path.join(PKG, "frontend", "md_js.cpp")
FRONTEND_BIN = os.path.join(OUT, "md_js")


def build_frontend(duktape_dir: str) -> str:
    """The script front end (frontend/md_js.cpp) linked against libfemmd.so,
    with the Duktape engine compiled from duktape_dir (duktape.cpp,
    duktape.h, duk_config.h: third-party sources this repository does not
    carry).  Returns the binary's path."""
    for f in ("duktape.cpp", "duktape.h", "duk_config.h"):
        if not os.path.exists(os.path.join(duktape_dir, f)):
            raise FileNotFoundError(os.path.join(duktape_dir, f))
    os.makedirs(OUT, exist_ok=True)
    engine = os.path.join(OUT, "duktape.o")
    cxx = os.environ.get("CXX", "g++")

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("front end build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)

    if _stale(engine, [os.path.join(duktape_dir, "duktape.cpp")]):
        run([cxx, "-O2", "-w", "-c", os.path.join(duktape_dir, "duktape.cpp"), "-I" + duktape_dir, "-o", engine])
    if _stale(FRONTEND_BIN, [FRONTEND, engine, LIB, os.path.join(ROOT, "include", "femmd.h")]):
        run([cxx, "-O2", "-std=c++17", "-Wall", FRONTEND, engine, "-I" + duktape_dir,
             "-I" + os.path.join(ROOT, "include"), "-L" + PKG, "-lfemmd", "-Wl,-rpath," + PKG, "-lm",
             "-o", FRONTEND_BIN])
    # where the engine came from (scripts shipped beside it are the tests' inputs)
    with open(FRONTEND_BIN + ".src", "w") as f:
        f.write(os.path.abspath(duktape_dir) + "\n")
    return FRONTEND_BIN


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
