"""GPU parity tests of the BN254 prove path (Config::field_type = BN254) through the C ABI.

Every BN254 golden case (digests of the reference prover templates instantiated over the
BN254 field, generated by tests/golden/make_golden.py) must be reproduced byte for byte:
proof bytes, claimed values and evaluated layers.  Exact integer arithmetic: the tolerance
is zero.
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
BN = GOLDEN["bn254_cases"]
M31 = GOLDEN["cases"]


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


@pytest.mark.parametrize("name", sorted(BN))
def test_bn254_proof_matches_reference_golden(ctx, name):
    g = BN[name]
    circ, w, grind = cases.build_bn(name)
    dc = ctx.load(circ, "BN254")
    cv, proof = ctx.prove(dc, w, grinding_bits=grind)
    assert cv.shape == (1, w.shape[1], 4)
    assert len(proof) == g["proof_len"]
    assert sha(proof) == g["proof_sha256"]
    assert sha(np.ascontiguousarray(cv).tobytes()) == g["claimed_v_sha256"]


@pytest.mark.parametrize("name", sorted(BN))
def test_bn254_evaluate_matches_reference_golden(ctx, name):
    g = BN[name]
    circ, w, _ = cases.build_bn(name)
    dc = ctx.load(circ, "BN254")
    assert sha(ctx.evaluate(dc, w).tobytes()) == g["output_sha256"]
    assert sha(ctx.evaluate(dc, w, all_layers=True).tobytes()) == g["values_sha256"]


@pytest.fixture(scope="module")
def obn():
    from oracle.oracle import OracleBn254
    return OracleBn254()


@pytest.mark.parametrize("seed,widths,n", [
    (401, [9, 11, 9, 11], 64), (402, [12, 10, 12], 16), (403, [2, 9, 3, 10, 1], 32),
    (404, [10, 10, 10], 7), (405, [11, 9], 100), (406, [8, 8, 8, 8], 1),
])
def test_bn254_gpu_matches_oracle_random(ctx, obn, seed, widths, n):
    """Random wiring at sizes beyond the goldens (and copy counts the reference driver is not
    instantiated for) against the C restatement, which the goldens pin."""
    circ = gc.random_circuit(seed, widths, p_mul=0.6, p_local=0.8, window=256)
    w = gc.random_witness_bn254(seed, circ.log_input_size, n)
    cv, proof = ctx.prove(ctx.load(circ, "BN254"), w)
    ocv, oproof = obn.prove(circ, w)
    assert proof == oproof
    assert np.array_equal(cv, ocv)
    assert obn.verify(circ, w, cv, proof)


def test_bn254_prover_api_mirror(ctx):
    from gkr_gb300.prover import Config, Proof, Prover
    cfg = Config(grinding_bits=10, field_type="BN254")
    assert cfg.get_num_repetitions() == 1
    circ, w, _ = cases.build_bn("bn_mixed_widths_n16")
    prover = Prover(cfg, ctx)
    prover.prepare_mem(circ)
    cv, proof = prover.prove(circ, w)
    assert isinstance(proof, Proof)
    assert sha(proof.bytes) == BN["bn_mixed_widths_n16"]["proof_sha256"]


def test_bn254_non_canonical_input_is_rejected(ctx):
    from gkr_gb300._lib import ERR_INVALID, GkrGpuError
    circ, w, g = cases.build_bn("bn_gkr_test_shape_n8")
    dc = ctx.load(circ, "BN254")
    bad = w.copy()
    r = [gc.BN254_R >> (64 * k) & (2**64 - 1) for k in range(4)]
    bad[3, 5, :] = np.array(r, np.uint64)  # exactly r
    with pytest.raises(GkrGpuError) as e:
        ctx.prove(dc, bad, grinding_bits=g)
    assert e.value.code == ERR_INVALID
    with pytest.raises(GkrGpuError):
        ctx.evaluate(dc, bad)
    # the context stays usable
    _, proof = ctx.prove(dc, w, grinding_bits=g)
    assert sha(proof) == BN["bn_gkr_test_shape_n8"]["proof_sha256"]


def test_bn254_and_m31_jobs_interleaved_in_lanes():
    """BN254 and M31 proofs queued together on a multi-lane context: every proof must still
    reproduce its golden, whatever completes first."""
    from gkr_gb300.prover import Context
    ctx = Context(0)
    try:
        ctx.set_concurrency(lanes=4)
        jobs = []
        for name in ["bn_lanes64", "cfg1_n16", "bn_full_coefs_n8", "lanes256", "bn_grind12_n16", "bn_edge_values_n8"]:
            if name.startswith("bn_"):
                c, w, g = cases.build_bn(name)
                dc = ctx.load(c, "BN254")
                cb = np.empty((1, w.shape[1], 4), np.uint64)
                gold = BN[name]
            else:
                c, w, g = cases.build(name)
                dc = ctx.load(c)
                cb = np.empty((3, w.shape[1]), np.uint32)
                gold = M31[name]
            pb = np.empty(dc.proof_size(w.shape[1], g), np.uint8)
            jobs.append((name, gold, ctx.submit(dc, w, pb, cb, grinding_bits=g), pb, cb, dc))
        for name, gold, job, pb, cb, _ in jobs:
            n = ctx.wait(job)
            assert sha(pb[:n].tobytes()) == gold["proof_sha256"], name
            assert sha(cb.tobytes()) == gold["claimed_v_sha256"], name
    finally:
        ctx.close()


def test_bn254_device_input(ctx):
    from gkr_gb300.prover import DeviceBuffer
    circ, w, g = cases.build_bn("bn_lanes64")
    dc = ctx.load(circ, "BN254")
    d = DeviceBuffer(ctx, w.nbytes)
    d.upload(w)
    pb = np.empty(dc.proof_size(64, g), np.uint8)
    cv, n = ctx.prove_device(dc, d.ptr, 64, pb, grinding_bits=g)
    assert sha(pb[:n].tobytes()) == BN["bn_lanes64"]["proof_sha256"]
    assert sha(np.ascontiguousarray(cv).tobytes()) == BN["bn_lanes64"]["claimed_v_sha256"]


@pytest.mark.parametrize("tile", [1, 8, 64, 256])
def test_bn254_row_tiles_do_not_change_proofs(tile):
    from gkr_gb300.prover import Context
    ctx = Context(0)
    try:
        ctx.set_tile(threads_per_row=tile)
        for name in ["bn_lanes64", "bn_mixed_widths_n16", "bn_width_one_n4"]:
            circ, w, g = cases.build_bn(name)
            _, proof = ctx.prove(ctx.load(circ, "BN254"), w, grinding_bits=g)
            assert sha(proof) == BN[name]["proof_sha256"], (tile, name)
    finally:
        ctx.close()


def test_host_buffer_views_keep_the_pinned_block_alive(ctx):
    import gc as pygc

    from gkr_gb300.prover import HostBuffer
    a = HostBuffer(1 << 16, np.uint64).array
    pygc.collect()
    a[:] = 7
    assert int(a.sum()) == 7 * (1 << 13)
