#!/bin/sh
# Builds oracle/_ref/libgkr_ref.so: the unmodified reference prover/verifier (header-only
# templates plus its vendored Bitcoin-Core SHA-256) behind oracle/ref_driver.cpp.
# Test infrastructure only; x86-64 with AVX-512 (the reference's own flags,
# CMakeLists.txt:9-12).  -DDISABLE_OPTIMIZED_SHA256 keeps the generic SHA-256 transform,
# which is the one the reference uses (its SSE4/AVX2/SHA-NI sources are not vendored).
# Usage: oracle/build_ref.sh REFERENCE_ROOT   (or GKR_REFERENCE_ROOT in the environment)
set -e
REF=${1:-$GKR_REFERENCE_ROOT}
[ -n "$REF" ] || { echo "usage: $0 REFERENCE_ROOT (or set GKR_REFERENCE_ROOT)" >&2; exit 2; }
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -d "$REF/include/LinearGKR" ] || { echo "reference tree not found at $REF" >&2; exit 3; }
case "$(uname -m)" in x86_64) ;; *) echo "reference build needs x86-64 AVX-512 (this is $(uname -m))" >&2; exit 4;; esac
mkdir -p "$OUT"
g++ -std=c++20 -O3 -march=native -mavx512f -mavx512vl -faligned-new -fPIC -shared -w \
    -DDISABLE_OPTIMIZED_SHA256 -DNDEBUG -I"$HERE" \
    -I"$REF/include" -I"$REF/lib" -I"$REF/lib/btc_sha256" \
    "$HERE/ref_driver.cpp" "$REF/lib/btc_sha256/crypto/sha256.cpp" \
    -o "$OUT/libgkr_ref.so.tmp"
mv "$OUT/libgkr_ref.so.tmp" "$OUT/libgkr_ref.so"
echo "built $OUT/libgkr_ref.so"
