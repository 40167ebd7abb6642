"""The C++ drop-in adapter (include/gkrgpu.hpp) compiles against the reference's own headers
and links against libgkrgpu.so: the reference's GKR_WITH_PC_TEST body builds with only the
prover type swapped.  Needs the reference tree, named by the environment variable
GKR_REFERENCE_ROOT (x86-64: the reference's SIMD build needs AVX-512)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("GKR_REFERENCE_ROOT", "")


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "include", "LinearGKR"))
                    or os.uname().machine != "x86_64",
                    reason="reference tree (GKR_REFERENCE_ROOT, x86-64 SIMD build) not available")
def test_adapter_builds_against_reference(tmp_path):
    from gkr_gb300 import build
    lib = build.build()
    exe = tmp_path / "gkr_test_with_adapter"
    cmd = ["g++", "-std=c++20", "-O1", "-march=native", "-mavx512f", "-mavx512vl", "-faligned-new", "-w",
           "-DDISABLE_OPTIMIZED_SHA256", f"-I{REF}/include", f"-I{REF}/lib", f"-I{REF}/lib/btc_sha256",
           f"-I{ROOT}/include", os.path.join(ROOT, "tests", "adapter", "gkr_test_with_adapter.cpp"),
           f"{REF}/lib/btc_sha256/crypto/sha256.cpp", lib, f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", str(exe)]
    subprocess.check_call(cmd)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    # 0: proved on a GPU, identical to the reference and verified; 77: no GPU on this machine
    assert r.returncode in (0, 77), r.stdout + r.stderr
