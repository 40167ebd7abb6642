"""Build recipe for the oracle (test infrastructure only).

``build_oracle()`` compiles the C restatement into ``oracle/build/libgkr_oracle.so``
with plain ``gcc -O3`` (portable: no -march flags, builds on x86-64 and aarch64).
``build_ref()`` runs ``oracle/build_ref.sh`` when the reference tree exists; its location
comes from the environment variable GKR_REFERENCE_ROOT (no default: without it the compiled
reference is simply not built, and the tests that need it skip).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
ORACLE_SO = os.path.join(BUILD, "libgkr_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libgkr_ref.so")


def reference_root():
    """The reference checkout named by GKR_REFERENCE_ROOT, or None."""
    root = os.environ.get("GKR_REFERENCE_ROOT", "")
    return root if root and os.path.isdir(os.path.join(root, "include", "LinearGKR")) else None


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    srcs = [os.path.join(HERE, f) for f in ("gkr_oracle.c", "gkr_oracle_bn254.c", "fs_hash.c", "gkr_oracle.h",
                                            "bn254.h")]
    if not force and not _stale(ORACLE_SO, srcs):
        return ORACLE_SO
    os.makedirs(BUILD, exist_ok=True)
    tmp = ORACLE_SO + ".tmp"
    subprocess.check_call(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread", "-Wall",
                           srcs[0], srcs[1], srcs[2], "-o", tmp])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(force=False):
    """Compile the reference driver (x86-64 only, needs the reference tree)."""
    root = reference_root()
    if root is None:
        return REF_SO if os.path.exists(REF_SO) and os.uname().machine == "x86_64" else None
    if os.uname().machine != "x86_64":
        return None
    srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "build_ref.sh"), os.path.join(HERE, "bn254.h")]
    if not force and not _stale(REF_SO, srcs):
        return REF_SO
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), root])
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
