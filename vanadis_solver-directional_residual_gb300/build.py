"""In-tree build of libvdr.so for sm_103a with nvcc (no cmake, no torch
extension machinery): one object per translation unit, compiled in
parallel, linked into ``lib/libvdr.so`` next to this file."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(LIB_DIR, "libvdr.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["element.cu", "apply.cu", "half.cu", "krylov.cu", "abi.cu", "noalloc.cu",
           "block.cu", "block_tc.cu", "unet.cu", "gcr.cu", "batch.cu", "tune.cu", "txtio.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required")
    return path


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
          if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "vdr.h"))
    return hs


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra_flags, "-I", CSRC,
                   "-I", INCLUDE, "-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for out in ex.map(run, jobs):
            if verbose and out:
                print(out)
    if force or jobs or _stale(LIB_PATH, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB_PATH, *objs,
               "-Xcompiler", "-fPIC"]
        run(cmd)
    return LIB_PATH
