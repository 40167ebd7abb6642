"""Builds libgkrgpu.so in-tree from csrc/ (nvcc for sm_103a, host C++ with the system compiler).

Three translation units are compiled in parallel and linked with nvcc; the CUDA runtime
is linked statically so the library only needs the driver at run time.
"""
import os
import platform
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
LIB = os.path.join(PKG, "libgkrgpu.so")
OBJ = os.path.join(ROOT, "_build")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O3", "-fPIC", "-std=c++17", "-Wall"]
if platform.machine() in ("aarch64", "arm64"):
    # ARMv8 SHA-2 instructions for the transcript hash (all Neoverse cores have them).
    CXXFLAGS.append("-march=armv8.2-a+crypto")

SOURCES = ["kernels.cu", "prover.cu", "sha256.cpp", "noalloc.cu", "bn254.cu", "circuit2.cpp", "keccak.cpp"]
HEADERS = ["kernels.cuh", "m31.cuh", "sha256.hpp", "transcript.hpp", "bn254.cuh", "bn254_prover.cuh", "fr_host.hpp",
           "verifier.cuh", "keccak.hpp"]


def _deps():
    return [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(INCLUDE, "gkrgpu.h"), __file__]


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def _cmd(src, obj):
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        return [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                "-Xcompiler", ",".join(CXXFLAGS), "-I", INCLUDE, "-c", path, "-o", obj]
    return [os.environ.get("CXX", "g++"), *CXXFLAGS, "-I", INCLUDE, "-c", path, "-o", obj]


def build(force=False, verbose=False):
    if not force and not needs_build():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(OBJ, src + ".o")
        objs.append(obj)
        cmd = _cmd(src, obj)
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"--- {src}\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if errors:
        raise RuntimeError("libgkrgpu build failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    subprocess.check_call([NVCC, *ARCH, "-shared", "-cudart", "static", *objs, "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
