"""In-tree build of libmaestro_adv.so for sm_103a (no cmake, no pip install).

Each CUDA translation unit is compiled in parallel, then linked into one shared library
next to this file.  ``--fmad=false`` (device code) and ``-ffp-contract=off`` (host code: the 1-D base-state
edges are formed on the host, and Arm compilers contract a*b+c into an FMA by default)
keep every floating-point expression as written, which is what makes the results
bit-identical to the reference algorithm evaluated in IEEE binary64.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmaestro_adv.so")
SOURCES = ["madv_kernels.cu", "madv_ctx.cu", "madv_probe.cu", "madv_box.cu", "madv_noalloc.cu", "madv_amr.cu", "madv_adjoint.cu", "madv_sphr.cu", "madv_macproj.cu", "madv_sweep.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def build_library(force=False, verbose=False):
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".hpp"))]
    deps.append(os.path.join(HERE, "..", "include", "maestro_adv.h"))
    deps.append(os.path.abspath(__file__))  # the source list and flags
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    procs, objs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        cmd = [nvcc()] + ARCH + FLAGS + ["-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd) + "\n" + out.decode())
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed: " + r.stdout.decode())
    os.replace(tmp, LIB)
    return LIB
