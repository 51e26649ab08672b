"""In-tree build of libsequoia_gpu.so (CUDA, sm_103a) and the host drop-in.

Every .cu file under csrc/ and every .cpp file under host/ (except the
command line tool) is compiled to an object in parallel and linked into
sequoia_gb300/libsequoia_gpu.so; host/sequoia_main.cpp becomes the
`sequoia_gb300/sequoia` executable linked against it.  Floating point:
-fmad=false and IEEE division / square root on the device, -ffp-contract=off
on the host, so the library's arithmetic is the oracle's operation for
operation.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
CLI_SRC = os.path.join(HOST, "sequoia_main.cpp")
CLI = os.path.join(HERE, "sequoia")
OUT_DIR = os.path.join(ROOT, "_build")
LIB = os.path.join(HERE, "libsequoia_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-Wall",
             "-I" + os.path.join(ROOT, "include"), "-I" + HOST]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def cxx():
    exe = shutil.which("g++") or shutil.which("c++")
    if not exe:
        raise RuntimeError("g++ not found")
    return exe


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def host_sources():
    return sorted(os.path.join(HOST, f) for f in os.listdir(HOST)
                  if f.endswith(".cpp") and os.path.join(HOST, f) != CLI_SRC)


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_flags=()):
    """Compile the CUDA library; returns the path of libsequoia_gpu.so."""
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "sequoia_gpu.h"))
    host_headers = [os.path.join(ROOT, "include", "sequoia_gpu.h"), os.path.join(ROOT, "include", "sequoia_host.h"),
                    *(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith((".hpp", ".h")))]
    procs, objs = [], []
    jobs = [(src, os.path.join(OUT_DIR, os.path.basename(src)[:-3] + ".o"), [nvcc(), *NVCC_FLAGS, *extra_flags],
             headers) for src in sources()]
    jobs += [(src, os.path.join(OUT_DIR, "host_" + os.path.basename(src)[:-4] + ".o"), [cxx(), *CXX_FLAGS],
              host_headers) for src in host_sources()]
    for src, obj, compiler, deps in jobs:
        objs.append(obj)
        if not _stale(obj, [src, *deps]):
            continue
        cmd = [*compiler, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if failed:
        msg = "\n".join("%s:\n%s" % f for f in failed)
        raise RuntimeError("compilation failed:\n" + msg)
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"]
        subprocess.run(cmd, check=True)
    if _stale(CLI, [LIB, CLI_SRC, *host_headers]):
        cmd = [cxx(), *CXX_FLAGS, CLI_SRC, "-o", CLI, "-L" + HERE, "-lsequoia_gpu", "-Wl,-rpath,$ORIGIN"]
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
