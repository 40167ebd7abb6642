"""Generates tests/golden/golden.json from the compiled, unmodified reference prover.

For every case of tests/cases.py it runs the reference Prover::prove (oracle/_ref, built
from the reference tree by oracle/build_ref.sh; the VectorizedM31 SIMD type at 8 copies,
the N-lane LaneVec type otherwise) and records SHA-256 digests of the proof bytes, of the
claimed values and of Circuit::evaluate's output, plus the proof length.  It also checks
that the reference verifier accepts the proof.  Run from the repository root:

    python tests/golden/make_golden.py
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


def main():
    obuild.build_ref()
    ref = Reference()
    out = {"generator": "reference Prover::prove via oracle/_ref (VectorizedM31 at 8 copies)", "cases": {}}
    for name in cases.CASES:
        circ, w, grind = cases.build(name)
        native = w.shape[1] == 8
        cv, proof = ref.prove(circ, w, grinding_bits=grind, native=native)
        assert ref.verify(circ, w, cv, proof, grinding_bits=grind, native=native), name
        ev = ref.evaluate(circ, w, native=native)
        out["cases"][name] = {
            "n_copies": int(w.shape[1]),
            "grinding_bits": grind,
            "proof_len": len(proof),
            "proof_sha256": digest(proof),
            "claimed_v_sha256": digest(np.ascontiguousarray(cv).tobytes()),
            "output_sha256": digest(np.ascontiguousarray(ev[-1]).tobytes()),
            "values_sha256": digest(np.concatenate(ev).tobytes()),
        }
        print(name, len(proof), out["cases"][name]["proof_sha256"][:16])
    # BN254: the reference templates over oracle/bn254.h's field (R = 1)
    bn = ReferenceBn254()
    out["bn254_generator"] = "reference Prover::prove templates over BN254 via oracle/_ref (N-lane LaneVec)"
    out["bn254_cases"] = {}
    for name in cases.BN_CASES:
        circ, w, grind = cases.build_bn(name)
        cv, proof = bn.prove(circ, w, grinding_bits=grind)
        assert bn.verify(circ, w, cv, proof, grinding_bits=grind), name
        ev = bn.evaluate(circ, w)
        out["bn254_cases"][name] = {
            "n_copies": int(w.shape[1]),
            "grinding_bits": grind,
            "proof_len": len(proof),
            "proof_sha256": digest(proof),
            "claimed_v_sha256": digest(np.ascontiguousarray(cv).tobytes()),
            "output_sha256": digest(np.ascontiguousarray(ev[-1]).tobytes()),
            "values_sha256": digest(np.concatenate(ev).tobytes()),
        }
        print(name, len(proof), out["bn254_cases"][name]["proof_sha256"][:16])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
