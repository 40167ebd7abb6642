"""CPU tests of the oracle: pinned to the reference's own outputs.

* golden.json holds digests of proofs made by the compiled, unmodified reference prover
  (tests/golden/make_golden.py); the C restatement must reproduce every one of them.
* Where the compiled reference is available, extra seeded cases are compared byte for
  byte, its VectorizedM31 SIMD path against the N-lane type, and both verifiers are run
  on honest and tampered proofs (tests/GKR_Test.cpp:30-31,63-78, tests/sumcheck.cpp:53-68).
"""
import hashlib
import json
import os

import numpy as np
import pytest

import cases
from gkr_gb300 import circuit as gc

_ALL = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
GOLDEN = _ALL["cases"]
LARGE = _ALL.get("large_cases", {})


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


@pytest.mark.parametrize("n", [0, 1, 31, 32, 55, 56, 57, 63, 64, 65, 119, 120, 1000, 12288])
def test_sha256_matches_hashlib(oracle, n):
    data = bytes((i * 131 + 7) & 0xFF for i in range(n))
    assert oracle.sha256(data) == hashlib.sha256(data).digest()


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_oracle_reproduces_reference_golden(oracle, name):
    g = GOLDEN[name]
    circ, w, grind = cases.build(name)
    cv, proof = oracle.prove(circ, w, grinding_bits=grind)
    assert len(proof) == g["proof_len"] == gc.Circuit.proof_size(circ, w.shape[1])
    assert sha(proof) == g["proof_sha256"]
    assert sha(cv.tobytes()) == g["claimed_v_sha256"]
    ev = oracle.evaluate(circ, w)
    assert sha(ev[-1].tobytes()) == g["output_sha256"]
    assert sha(np.concatenate(ev).tobytes()) == g["values_sha256"]
    assert oracle.verify(circ, w, cv, proof, grinding_bits=grind)


def test_oracle_reproduces_reference_golden_config2(oracle):
    """The benchmark's config-2 circuit (24 layers alternating 2^18 / 2^20 gates) at 8
    copies: the restatement reproduces the compiled reference's proof byte for byte."""
    name = "cfg2_n8"
    g = LARGE[name]
    circ, w, grind = cases.build(name)
    cv, proof = oracle.prove(circ, w, grinding_bits=grind)
    assert len(proof) == g["proof_len"]
    assert sha(proof) == g["proof_sha256"]
    assert sha(cv.tobytes()) == g["claimed_v_sha256"]


def test_oracle_rejects_tampering(oracle):
    circ, w, grind = cases.build("cfg1_n16")
    cv, proof = oracle.prove(circ, w)
    N = w.shape[1]
    com = (1 << circ.log_input_size) * N * 4 + 32
    for pos in [com + 5, com + 12 * N + 3, len(proof) - 1, len(proof) // 2]:
        bad = bytearray(proof)
        bad[pos] ^= 0x01
        assert not oracle.verify(circ, w, cv, bytes(bad)), pos
    bad_cv = cv.copy()
    bad_cv[1, 3] = (int(bad_cv[1, 3]) + 1) % gc.P
    assert not oracle.verify(circ, w, bad_cv, proof)
    assert not oracle.verify(circ, w, cv, proof[:-4])


def test_eval_multilinear_matches_definition(oracle):
    st = gc.Stream(3)
    evals = st.field(32 * 4).reshape(32, 4)
    r = st.field(5)
    got = oracle.eval_multilinear(evals, r)
    # direct sum_z eq(r, z) evals[z] with python ints
    P = gc.P
    want = [0] * 4
    for z in range(32):
        e = 1
        for t in range(5):
            e = e * (int(r[t]) if (z >> t) & 1 else (1 - int(r[t])) % P) % P
        for k in range(4):
            want[k] = (want[k] + e * int(evals[z, k])) % P
    assert list(got) == want


# ---------------------------------------------------------------- against the compiled reference

@pytest.mark.parametrize("seed,widths,n", [
    (101, [4, 4, 4, 4], 4), (102, [5, 3, 6, 2], 8), (103, [2, 6, 1, 3], 16), (104, [7, 7], 32),
    (105, [3, 3, 3, 3, 3, 3, 3], 8), (106, [6, 8, 6], 64), (107, [1, 4, 1], 48), (108, [4, 0], 16),
])
def test_oracle_matches_reference(oracle, reference, seed, widths, n):
    circ = gc.random_circuit(seed, widths, p_mul=0.5, p_local=0.5, window=4)
    w = gc.random_witness(seed, circ.log_input_size, n)
    rcv, rproof = reference.prove(circ, w)
    ocv, oproof = oracle.prove(circ, w)
    assert oproof == rproof
    assert np.array_equal(ocv, rcv)
    ev_r, ev_o = reference.evaluate(circ, w), oracle.evaluate(circ, w)
    assert all(np.array_equal(a, b) for a, b in zip(ev_r, ev_o))


def test_reference_simd_path_equals_lane_type(reference):
    circ, w, grind = cases.build("cfg1_n8")
    a = reference.prove(circ, w, native=True)
    b = reference.prove(circ, w, native=False)
    assert a[1] == b[1] and np.array_equal(a[0], b[0])


def test_verifiers_agree_on_tampering(oracle, reference):
    circ, w, grind = cases.build("mixed_widths_n16")
    cv, proof = oracle.prove(circ, w)
    assert reference.verify(circ, w, cv, proof)
    st = gc.Stream(9)
    for pos in st.below(12, len(proof) - 32 * 0).tolist():
        bad = bytearray(proof)
        bad[int(pos)] ^= 0x40
        r = reference.verify(circ, w, cv, bytes(bad))
        o = oracle.verify(circ, w, cv, bytes(bad))
        assert r == o
