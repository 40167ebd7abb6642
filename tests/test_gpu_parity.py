"""GPU parity tests: proofs from the CUDA path through the C ABI against the reference.

Every golden case (digests of the compiled, unmodified reference prover's output) must be
reproduced byte for byte (proof bytes, claimed values, evaluated layers), the oracle's
restated verifier must accept the GPU proof, and tampering must be rejected.  Exact
integer arithmetic: the tolerance is zero.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import cases
from gkr_gb300 import circuit as gc

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["cases"]


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_gpu_proof_matches_reference_golden(ctx, oracle, name):
    g = GOLDEN[name]
    circ, w, grind = cases.build(name)
    dc = ctx.load(circ)
    cv, proof = ctx.prove(dc, w, grinding_bits=grind)
    assert len(proof) == g["proof_len"]
    assert sha(proof) == g["proof_sha256"]
    assert sha(np.ascontiguousarray(cv).tobytes()) == g["claimed_v_sha256"]
    assert oracle.verify(circ, w, cv, proof, grinding_bits=grind)


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_gpu_evaluate_matches_reference_golden(ctx, name):
    g = GOLDEN[name]
    circ, w, _ = cases.build(name)
    dc = ctx.load(circ)
    assert sha(ctx.evaluate(dc, w).tobytes()) == g["output_sha256"]
    assert sha(ctx.evaluate(dc, w, all_layers=True).tobytes()) == g["values_sha256"]


@pytest.mark.parametrize("seed,widths,n", [
    (201, [9, 11, 9, 11], 64), (202, [12, 10, 12], 16), (203, [8, 8, 8, 8, 8, 8], 128),
    (204, [2, 9, 3, 10, 1], 32), (205, [13, 11], 8), (206, [10, 12, 10], 1024),
])
def test_gpu_matches_oracle_random(ctx, oracle, seed, widths, n):
    circ = gc.random_circuit(seed, widths, p_mul=0.6, p_local=0.8, window=256)
    w = gc.random_witness(seed, circ.log_input_size, n)
    cv, proof = ctx.prove(ctx.load(circ), w)
    ocv, oproof = oracle.prove(circ, w)
    assert proof == oproof
    assert np.array_equal(cv, ocv)


def test_gpu_proof_tamper_rejected(ctx, oracle):
    circ, w, grind = cases.build("cfg1_n16")
    cv, proof = ctx.prove(ctx.load(circ), w)
    N = w.shape[1]
    com = (1 << circ.log_input_size) * N * 4 + 32
    for pos in [com + 7, com + 24 * N + 1, len(proof) - 2]:
        bad = bytearray(proof)
        bad[pos] ^= 0x10
        assert not oracle.verify(circ, w, cv, bytes(bad))
    bad_cv = cv.copy()
    bad_cv[0, 0] = (int(bad_cv[0, 0]) + 1) % gc.P
    assert not oracle.verify(circ, w, bad_cv, proof)


def test_repeated_proofs_identical_and_context_reuse(ctx):
    # workspace reuse across circuits of different shapes and copy counts
    a = cases.build("cfg1_n16")
    b = cases.build("lanes1024")
    da, db = ctx.load(a[0]), ctx.load(b[0])
    pa1 = ctx.prove(da, a[1])[1]
    pb1 = ctx.prove(db, b[1])[1]
    pa2 = ctx.prove(da, a[1])[1]
    pb2 = ctx.prove(db, b[1])[1]
    assert pa1 == pa2 and pb1 == pb2


def test_non_canonical_input_is_rejected(ctx):
    from gkr_gb300._lib import GkrGpuError
    circ, w, _ = cases.build("cfg1_n16")
    w = w.copy()
    w[3, 5] = gc.P
    with pytest.raises(GkrGpuError):
        ctx.prove(ctx.load(circ), w)


def test_bad_lane_count_is_rejected(ctx):
    from gkr_gb300._lib import GkrGpuError
    circ = gc.random_circuit(1, [4, 4])
    w = gc.random_witness(1, 4, 6)
    with pytest.raises(GkrGpuError):
        ctx.prove(ctx.load(circ), w)


def test_prover_api_mirror(ctx, oracle):
    from gkr_gb300.prover import Config, Proof, Prover
    circ, w, _ = cases.build("gkr_test_shape_n16")
    circ.set_input(w)
    prover = Prover(Config(), ctx)
    prover.prepare_mem(circ)
    cv, proof = prover.prove(circ)
    assert isinstance(proof, Proof)
    assert sha(proof.bytes) == GOLDEN["gkr_test_shape_n16"]["proof_sha256"]
    assert oracle.verify(circ, w, cv, proof.bytes)
