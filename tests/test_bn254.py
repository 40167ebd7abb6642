"""CPU tests of the BN254 field definition (oracle/bn254.h) against Python integers, and of
the reference templates instantiated with it (prove -> verify round trips, tampering)."""
import numpy as np
import pytest

from gkr_gb300 import circuit as gc

R = gc.BN254_R


@pytest.fixture(scope="module")
def refbn():
    from oracle.oracle import Reference, ReferenceBn254
    if not Reference.available():
        pytest.skip("compiled reference (oracle/_ref) not available on this machine")
    return ReferenceBn254()


def test_field_ops_match_python_integers(refbn):
    st = gc.Stream(4)
    vals = [int(x) % R for x in gc.bn254_values(gc.random_witness_bn254(4, 4, 8))]
    edge = [0, 1, 2, R - 1, R - 2, (R + 1) // 2]
    for a, b in zip(vals + edge, list(reversed(vals)) + edge[::-1]):
        assert refbn.field_op("mul", a, b) == a * b % R
        assert refbn.field_op("add", a, b) == (a + b) % R
        assert refbn.field_op("sub", a, b) == (a - b) % R
    for x in [R, R + 5, 2**256 - 1, 5 * R, 5 * R + 7] + [int(v) for v in st.u64(8)]:
        assert refbn.field_op("reduce", x % 2**256) == (x % 2**256) % R


def test_witness_is_canonical():
    w = gc.random_witness_bn254(9, 6, 16)
    assert w.shape == (64, 16, 4)
    assert max(gc.bn254_values(w)) < R


def test_reference_templates_prove_and_verify_bn254(refbn):
    circ = gc.random_circuit(41, [5, 4, 5, 3], p_mul=0.5)
    w = gc.random_witness_bn254(41, circ.log_input_size, 16)
    cv, proof = refbn.prove(circ, w)
    assert len(proof) == refbn.proof_size(circ, 16)
    assert refbn.verify(circ, w, cv, proof)
    bad = bytearray(proof)
    bad[-40] ^= 1
    assert not refbn.verify(circ, w, cv, bytes(bad))
    ev = refbn.evaluate(circ, w)
    # spot-check one output lane of the first layer by Python integers
    l0 = circ.layers[0]
    out = [0] * (1 << l0.nb_output_vars)
    inp = [gc.bn254_values(w[i, 3])[0] for i in range(1 << l0.nb_input_vars)]
    for o, i0, i1, c in l0.mul.tolist():
        out[o] = (out[o] + inp[i0] * inp[i1] * c) % R
    for o, i0, c in l0.add.tolist():
        out[o] = (out[o] + inp[i0] * c) % R
    got = [gc.bn254_values(ev[1][i, 3])[0] for i in range(len(out))]
    assert got == out


# ---------------------------------------------------------------- the C restatement over BN254
import hashlib  # noqa: E402
import json  # noqa: E402
import os  # noqa: E402

import cases  # noqa: E402

GOLDEN_BN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["bn254_cases"]


@pytest.fixture(scope="module")
def obn():
    from oracle.oracle import OracleBn254
    return OracleBn254()


def _sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


@pytest.mark.parametrize("name", sorted(GOLDEN_BN))
def test_bn254_oracle_matches_reference_golden(obn, name):
    g = GOLDEN_BN[name]
    circ, w, grind = cases.build_bn(name)
    cv, proof = obn.prove(circ, w, grinding_bits=grind)
    assert len(proof) == g["proof_len"] == obn.proof_size(circ, w.shape[1])
    assert _sha(proof) == g["proof_sha256"]
    assert _sha(cv.tobytes()) == g["claimed_v_sha256"]
    assert _sha(np.concatenate(obn.evaluate(circ, w)).tobytes()) == g["values_sha256"]
    assert obn.verify(circ, w, cv, proof, grinding_bits=grind)


def test_bn254_oracle_rejects_tampering(obn):
    circ, w, grind = cases.build_bn("bn_mixed_widths_n16")
    cv, proof = obn.prove(circ, w, grinding_bits=grind)
    n0 = (1 << circ.log_input_size) * 16 * 32 + 32
    for pos in (n0 + 5, len(proof) // 2, len(proof) - 1):
        bad = bytearray(proof)
        bad[pos] ^= 0x10
        assert not obn.verify(circ, w, cv, bytes(bad), grinding_bits=grind), pos
    cv2 = cv.copy()
    cv2[0, 3, 0] ^= 1
    assert not obn.verify(circ, w, cv2, proof, grinding_bits=grind)
    assert not obn.verify(circ, w, cv, proof[:-32], grinding_bits=grind)


def test_bn254_oracle_rejects_non_canonical_input(obn):
    circ, w, grind = cases.build_bn("bn_width_one_n4")
    bad = w.copy()
    bad[1, 2, :] = np.array([R >> (64 * k) & (2**64 - 1) for k in range(4)], np.uint64)
    with pytest.raises(ValueError):
        obn.prove(circ, bad, grinding_bits=grind)


@pytest.mark.parametrize("seed,widths,n", [(301, [6, 7, 5, 6], 16), (302, [8, 6, 8], 4), (303, [5, 5, 5, 5], 64)])
def test_bn254_oracle_matches_reference_random(obn, refbn, seed, widths, n):
    circ = gc.random_circuit(seed, widths, p_mul=0.6, p_local=0.7, window=32)
    w = gc.random_witness_bn254(seed, circ.log_input_size, n)
    cv, proof = obn.prove(circ, w)
    rcv, rproof = refbn.prove(circ, w)
    assert proof == rproof
    assert np.array_equal(cv, rcv)
