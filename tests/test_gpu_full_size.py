"""GPU parity at the benchmark's own sizes.

* The config-2 circuit the benchmark times (24 layers alternating 2^18 / 2^20 gates, 60% mul,
  wiring local to 2^12-gate windows) and the config-4 BN254 circuit (16 layers of 2^16 gates)
  at the few copies the compiled reference proves in seconds: proof bytes, claimed values and
  every evaluated layer must equal the reference's digests (tests/golden/golden.json,
  "large_cases" / "bn254_large_cases"), with the library's default row tiles and with the
  tiles its autotuner picks for the 1024-copy proof.
* The 1024-copy config-2 proof itself (1 GiB of commitment, 2^20-row layers, the autotuned
  row loops and CTA budgets of the timed run) is too large for the CPU prover, so it is
  checked through size-independent properties: the oracle's restatement of the reference
  verifier accepts it and rejects it tampered, its commitment is the witness, and the
  default-tile proof and the autotuned proof are identical.
Exact integer arithmetic: the tolerance is zero.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import cases
from gkr_gb300 import circuit as gc

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
LARGE = GOLDEN.get("large_cases", {})
BN_LARGE = GOLDEN.get("bn254_large_cases", {})
N_FULL = 1024


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


@pytest.fixture(scope="module")
def config2():
    return gc.config2_circuit()


@pytest.fixture(scope="module")
def full(config2):
    """A context proving the 1024-copy config-2 proof with the autotuned tiles, the proof
    and its claims; closed at the end of the module (about 90 GiB of workspace)."""
    from gkr_gb300 import build as libbuild
    libbuild.build()
    from gkr_gb300.prover import Context
    ctx = Context(0)
    dc = ctx.load(config2)
    w = gc.random_witness(1000, config2.log_input_size, N_FULL)
    tiles = ctx.autotune(dc, w)
    cv, proof = ctx.prove(dc, w)
    yield {"ctx": ctx, "dc": dc, "w": w, "cv": cv, "proof": proof, "tiles": tiles}
    dc.free()
    ctx.close()


@pytest.mark.parametrize("name", sorted(LARGE))
@pytest.mark.parametrize("tiles", ["default", "autotuned"])
def test_config2_matches_reference_golden(ctx, full, config2, name, tiles):
    g = LARGE[name]
    circ, w, grind = cases.build(name)
    assert g["witness_seed"] == cases.witness_seed(name)
    c = full["ctx"] if tiles == "autotuned" else ctx
    dc = full["dc"] if tiles == "autotuned" else ctx.load(config2)
    cv, proof = c.prove(dc, w, grinding_bits=grind)
    assert len(proof) == g["proof_len"]
    assert sha(proof) == g["proof_sha256"]
    assert sha(np.ascontiguousarray(cv).tobytes()) == g["claimed_v_sha256"]
    if tiles == "default":
        assert sha(c.evaluate(dc, w, all_layers=True).tobytes()) == g["values_sha256"]


def test_config2_full_size_accepted_by_the_oracle_verifier(full, config2, oracle):
    proof, cv, w = full["proof"], full["cv"], full["w"]
    assert len(proof) == gc.Circuit.proof_size(config2, N_FULL)
    # RAW commitment: the input rows verbatim
    com = w.nbytes
    assert proof[:com] == w.tobytes()
    assert oracle.verify(config2, w, cv, proof)


def test_config2_full_size_tampered_is_rejected(full, config2, oracle):
    proof, cv, w = full["proof"], full["cv"], full["w"]
    bad = bytearray(proof)
    bad[len(bad) - 4 * N_FULL - 2] ^= 0x10  # a word of the first layer's last vy claim
    assert not oracle.verify(config2, w, cv, bytes(bad))


def test_config2_full_size_tiles_do_not_change_bytes(ctx, full, config2):
    cv, proof = ctx.prove(ctx.load(config2), full["w"])
    assert proof == full["proof"]
    assert np.array_equal(cv, full["cv"])


@pytest.mark.parametrize("name", sorted(BN_LARGE))
def test_config4_bn254_matches_reference_golden(ctx, name):
    g = BN_LARGE[name]
    circ, w, grind = cases.build_bn(name)
    assert g["witness_seed"] == cases.witness_seed(name)
    dc = ctx.load(circ, "BN254")
    cv, proof = ctx.prove(dc, w, grinding_bits=grind)
    assert len(proof) == g["proof_len"]
    assert sha(proof) == g["proof_sha256"]
    assert sha(np.ascontiguousarray(cv).tobytes()) == g["claimed_v_sha256"]
    assert sha(ctx.evaluate(dc, w, all_layers=True).tobytes()) == g["values_sha256"]
