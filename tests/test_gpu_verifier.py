"""GPU-assisted verifier (gkrgpu_verify) against the oracle's restatement of the reference
verifier: the same accept/reject decision on honest proofs, tampered proofs and claims, and
on the malleations the reference tolerates (grinding bytes it skips, trailing bytes it never
reads, non-canonical encodings it reduces)."""
import hashlib
import json
import os

import numpy as np
import pytest

import cases
from gkr_gb300 import circuit as gc

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["cases"]


@pytest.mark.parametrize("name", ["cfg1_n16", "gkr_test_shape_n8", "mixed_widths_n16", "output_scalar_n16",
                                  "lanes1024", "grind8_n16", "all_to_one_n8", "sparse_top_n32"])
def test_verifier_accepts_golden_proofs(ctx, name):
    circ, w, g = cases.build(name)
    dc = ctx.load(circ)
    cv, proof = ctx.prove(dc, w, grinding_bits=g)
    assert hashlib.sha256(proof).hexdigest() == GOLDEN[name]["proof_sha256"]
    assert ctx.verify(dc, proof, cv, grinding_bits=g)


def _flip(b, pos, bit=1):
    x = bytearray(b)
    x[pos] ^= bit
    return bytes(x)


def test_verifier_decisions_match_oracle(ctx, oracle):
    circ, w, g = cases.build("mixed_widths_n16")
    dc = ctx.load(circ)
    cv, proof = ctx.prove(dc, w, grinding_bits=g)
    N = w.shape[1]
    com = (1 << circ.log_input_size) * N * 4
    variants = {
        "honest": (proof, cv),
        "commitment": (_flip(proof, 5), cv),
        "first round": (_flip(proof, com + 32 + 7), cv),
        "middle": (_flip(proof, len(proof) // 2), cv),
        "last vy": (_flip(proof, len(proof) - 3), cv),
        "truncated": (proof[:-4], cv),
        "claim": (proof, cv ^ np.uint32(1) * (np.arange(cv.size).reshape(cv.shape) == 5)),
        "grinding bytes": (_flip(proof, com + 3), cv),
        "trailing bytes": (proof + b"\x01\x02\x03\x04", cv),
    }
    # a round value re-encoded as value + p (< 2^32) reads back as the same field element
    pos = com + 32 + 4 * 3
    v = int.from_bytes(proof[pos:pos + 4], "little")
    if v + gc.P < 2**32:
        variants["non-canonical encoding"] = (proof[:pos] + (v + gc.P).to_bytes(4, "little") + proof[pos + 4:], cv)
    for what, (pb, c) in variants.items():
        want = oracle.verify(circ, w, c, pb, grinding_bits=g)
        assert ctx.verify(dc, pb, c, grinding_bits=g) == want, what
    assert ctx.verify(dc, proof, cv, grinding_bits=g)
    assert not ctx.verify(dc, _flip(proof, len(proof) // 3), cv, grinding_bits=g)
    assert ctx.verify(dc, _flip(proof, com + 3), cv, grinding_bits=g)  # grinding bytes are not read


@pytest.mark.parametrize("seed,widths,n", [(501, [12, 10, 12, 11], 64), (502, [9, 13, 9], 256), (503, [14, 12], 16)])
def test_verifier_on_larger_circuits(ctx, oracle, seed, widths, n):
    from gkr_gb300.prover import Config, Verifier
    circ = gc.random_circuit(seed, widths, p_mul=0.6, p_local=0.8, window=256)
    w = gc.random_witness(seed, circ.log_input_size, n)
    dc = ctx.load(circ)
    cv, proof = ctx.prove(dc, w)
    assert Verifier(Config(), ctx).verify(circ, cv, proof)
    bad = cv.copy()
    bad[1, 0] = (int(bad[1, 0]) + 1) % gc.P
    assert not ctx.verify(dc, proof, bad)
    assert not oracle.verify(circ, w, bad, proof)


@pytest.mark.parametrize("name", ["bn_mixed_widths_n16", "bn_width_one_n4", "bn_full_coefs_n8", "bn_lanes64",
                                  "bn_grind0_n8"])
def test_bn254_verifier_decisions_match_oracle(ctx, name):
    from oracle.oracle import OracleBn254
    obn = OracleBn254()
    circ, w, g = cases.build_bn(name)
    dc = ctx.load(circ, "BN254")
    cv, proof = ctx.prove(dc, w, grinding_bits=g)
    N = w.shape[1]
    com = (1 << circ.log_input_size) * N * 32
    bad_cv = cv.copy()
    bad_cv[0, N - 1, 0] ^= np.uint64(2)
    variants = {
        "honest": (proof, cv),
        "commitment": (_flip(proof, 33), cv),
        "first round": (_flip(proof, com + 32 + 40), cv),
        "last vy": (_flip(proof, len(proof) - 5), cv),
        "truncated": (proof[:-32], cv),
        "claim": (proof, bad_cv),
        "grinding bytes": (_flip(proof, com + 9), cv),
        "trailing bytes": (proof + bytes(8), cv),
    }
    for what, (pb, c) in variants.items():
        want = obn.verify(circ, w, c, pb, grinding_bits=g)
        assert ctx.verify(dc, pb, c, grinding_bits=g) == want, what
    assert ctx.verify(dc, proof, cv, grinding_bits=g)
    assert not ctx.verify(dc, proof, bad_cv, grinding_bits=g)
