"""Generates tests/golden/golden.json from the compiled, unmodified reference prover.

For every case of tests/cases.py it runs the reference Prover::prove (oracle/_ref, built
from the reference tree by oracle/build_ref.sh; the VectorizedM31 SIMD type at 8 copies,
the N-lane LaneVec type otherwise) and records SHA-256 digests of the proof bytes, of the
claimed values and of Circuit::evaluate's output, plus the proof length.  It also checks
that the reference verifier accepts the proof.  Run from the repository root:

    python tests/golden/make_golden.py            # every section
    python tests/golden/make_golden.py large      # only the full-size benchmark circuits

The reference tree is found through the environment variable GKR_REFERENCE_ROOT.  The
large sections ("large_cases", "bn254_large_cases") hold the benchmark's own config-2 and
config-4 circuits at a few copies, with the witness seed of each case.
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "expander-cpp_gb300"), os.path.join(ROOT, "tests")]

import numpy as np  # noqa: E402

import cases  # noqa: E402
from oracle import build as obuild  # noqa: E402
from oracle.oracle import Reference, ReferenceBn254  # noqa: E402


def digest(b):
    return hashlib.sha256(bytes(b)).hexdigest()


def record(name, w, grind, cv, proof, ev):
    return {
        "n_copies": int(w.shape[1]),
        "grinding_bits": grind,
        "witness_seed": cases.witness_seed(name),
        "proof_len": len(proof),
        "proof_sha256": digest(proof),
        "claimed_v_sha256": digest(np.ascontiguousarray(cv).tobytes()),
        "output_sha256": digest(np.ascontiguousarray(ev[-1]).tobytes()),
        "values_sha256": digest(np.concatenate(ev).tobytes()),
    }


def m31_section(names):
    ref = Reference()
    sec = {}
    for name in names:
        circ, w, grind = cases.build(name)
        native = w.shape[1] == 8
        cv, proof = ref.prove(circ, w, grinding_bits=grind, native=native)
        assert ref.verify(circ, w, cv, proof, grinding_bits=grind, native=native), name
        ev = ref.evaluate(circ, w, native=native)
        sec[name] = record(name, w, grind, cv, proof, ev)
        print(name, len(proof), sec[name]["proof_sha256"][:16], flush=True)
    return sec


def bn254_section(names):
    # BN254: the reference templates over oracle/bn254.h's field (R = 1)
    bn = ReferenceBn254()
    sec = {}
    for name in names:
        circ, w, grind = cases.build_bn(name)
        cv, proof = bn.prove(circ, w, grinding_bits=grind)
        assert bn.verify(circ, w, cv, proof, grinding_bits=grind), name
        ev = bn.evaluate(circ, w)
        sec[name] = record(name, w, grind, cv, proof, ev)
        print(name, len(proof), sec[name]["proof_sha256"][:16], flush=True)
    return sec


def main():
    if obuild.build_ref() is None:
        raise SystemExit("the compiled reference is needed: set GKR_REFERENCE_ROOT to the reference tree (x86-64)")
    which = sys.argv[1:] or ["small", "large"]
    path = os.path.join(HERE, "golden.json")
    out = json.load(open(path)) if os.path.exists(path) else {}
    out["generator"] = "reference Prover::prove via oracle/_ref (VectorizedM31 at 8 copies)"
    out["bn254_generator"] = "reference Prover::prove templates over BN254 via oracle/_ref (N-lane LaneVec)"
    if "small" in which:
        out["cases"] = m31_section(cases.CASES)
        out["bn254_cases"] = bn254_section(cases.BN_CASES)
    if "large" in which:
        out["large_cases"] = m31_section(cases.LARGE_CASES)
        out["bn254_large_cases"] = bn254_section(cases.BN_LARGE_CASES)
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
