#!/usr/bin/env python3
"""Build the GB300 codec in-tree: libvc.so (vc.h / vcg.h C ABI, CUDA for
sm_103a + C host code) and libvcsynth.so (host synthetic-volume generator).

Usage: python build.py [--force]. Objects go to _build/ next to this file;
the shared libraries are written beside this file."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CC = os.environ.get("CC", "gcc")

CU_SRCS = ["vc_device.cu", "vc_encode.cu", "k_decode.cu", "k_encode.cu", "k_synth.cu", "vc_noalloc.cu", "k_batch.cu", "vc_batch.cu", "k_dct.cu", "k_repack.cu", "k_ds.cu"]
C_SRCS = ["vc_host.c", "vc_server.c", "vc_writer.c"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xptxas", "-O3",
                     "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off,-O2",
                     "-I" + SRC]
C_FLAGS = ["-std=gnu2x", "-O2", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-fno-fast-math",
           "-Wall", "-Wextra", "-I" + SRC]
LIB = os.path.join(HERE, "libvc.so")
SYNTH = os.path.join(HERE, "libvcsynth.so")


def newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def headers():
    return [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))] + \
        [os.path.join(HERE, "..", "include", "vc.h")]


def compile_one(src, force):
    path = os.path.join(SRC, src)
    obj = os.path.join(OBJ, src + ".o")
    if not force and not newer(obj, [path] + headers()):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC] + NVCC_FLAGS + ["-c", path, "-o", obj]
    else:
        cmd = [CC] + C_FLAGS + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(force=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = CU_SRCS + C_SRCS
    with ThreadPoolExecutor(len(srcs)) as ex:
        objs = list(ex.map(lambda s: compile_one(s, force), srcs))
    if force or newer(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread", "-lm"]
        subprocess.run(cmd, check=True)
    synth_src = os.path.join(SRC, "synth.c")
    if force or newer(SYNTH, [synth_src, os.path.join(SRC, "synth_core.h")]):
        subprocess.run([CC, "-std=gnu11", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                        "-fno-fast-math", "-fvisibility=hidden", "-o", SYNTH, synth_src, "-lm"], check=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("built", LIB, SYNTH)
