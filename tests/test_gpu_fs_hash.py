"""Proofs with the Keccak-256 transcript (gkrgpu_set_fs_hash) on the GPU against the oracle's
Keccak-mode proofs, byte for byte, for M31 and BN254; the GPU verifier accepts them in
Keccak mode and rejects them in SHA-256 mode.  Every test puts the context back to SHA-256."""
import hashlib
import json
import os

import pytest

import cases

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["cases"]


@pytest.fixture
def keccak(ctx, oracle):
    ctx.set_fs_hash("Keccak256")
    oracle.set_fs_hash("Keccak256")
    yield
    ctx.set_fs_hash("SHA256")
    oracle.set_fs_hash("SHA256")


@pytest.mark.parametrize("name", ["cfg1_n16", "mixed_widths_n16", "grind8_n16", "lanes1024", "output_scalar_n16"])
def test_m31_keccak_proofs_match_oracle(ctx, oracle, keccak, name):
    circ, w, g = cases.build(name)
    dc = ctx.load(circ)
    cv, proof = ctx.prove(dc, w, grinding_bits=g)
    want_cv, want = oracle.prove(circ, w, grinding_bits=g)
    assert proof == want
    assert (cv == want_cv).all()
    assert hashlib.sha256(proof).hexdigest() != GOLDEN[name]["proof_sha256"]
    assert ctx.verify(dc, proof, cv, grinding_bits=g)
    ctx.set_fs_hash("SHA256")
    assert not ctx.verify(dc, proof, cv, grinding_bits=g)


def test_m31_keccak_queued_proofs(ctx, oracle, keccak):
    """Proofs submitted through the asynchronous queue use the hash set when submitted."""
    import numpy as np
    from gkr_gb300.prover import HostBuffer
    circ, w, g = cases.build("mixed_widths_n16")
    dc = ctx.load(circ)
    N = w.shape[1]
    want_cv, want = oracle.prove(circ, w, grinding_bits=g)
    cap = dc.proof_size(N, g)
    bufs = [(HostBuffer(cap), HostBuffer(dc.num_repetitions(g) * N * 4, np.uint32)) for _ in range(3)]
    jobs = [ctx.submit(dc, w, pb.array, cb.array, grinding_bits=g) for pb, cb in bufs]
    for job, (pb, cb) in zip(jobs, bufs):
        n = ctx.wait(job)
        assert bytes(pb.array[:n]) == want


@pytest.mark.parametrize("name", ["bn_mixed_widths_n16", "bn_grind0_n8", "bn_lanes64"])
def test_bn254_keccak_proofs_match_oracle(ctx, keccak, name):
    from oracle.oracle import OracleBn254
    obn = OracleBn254()
    circ, w, g = cases.build_bn(name)
    dc = ctx.load(circ, "BN254")
    cv, proof = ctx.prove(dc, w, grinding_bits=g)
    want_cv, want = obn.prove(circ, w, grinding_bits=g)
    assert proof == want
    assert (cv == want_cv).all()
    assert ctx.verify(dc, proof, cv, grinding_bits=g)
    ctx.set_fs_hash("SHA256")
    assert not ctx.verify(dc, proof, cv, grinding_bits=g)


def test_prover_config_selects_hash(ctx, oracle):
    from gkr_gb300.prover import Config, Prover, Verifier
    circ, w, g = cases.build("cfg1_n16")
    circ.set_input(w)
    try:
        cv, proof = Prover(Config(g, FS_hash="Keccak256"), ctx).prove(circ)
        oracle.set_fs_hash("Keccak256")
        assert proof.bytes == oracle.prove(circ, w, grinding_bits=g)[1]
        assert Verifier(Config(g, FS_hash="Keccak256"), ctx).verify(circ, cv, proof)
        assert not Verifier(Config(g), ctx).verify(circ, cv, proof)
    finally:
        ctx.set_fs_hash("SHA256")
        oracle.set_fs_hash("SHA256")
