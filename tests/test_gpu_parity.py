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
    # row slices of 96 and 160 copies: the one-copy-per-thread kernels leave warps idle
    (207, [9, 10, 9], 96), (208, [8, 9, 8], 160),
])
def test_gpu_matches_oracle_random(ctx, oracle, seed, widths, n):
    circ = gc.random_circuit(seed, widths, p_mul=0.6, p_local=0.8, window=256)
    w = gc.random_witness(seed, circ.log_input_size, n)
    cv, proof = ctx.prove(ctx.load(circ), w)
    ocv, oproof = oracle.prove(circ, w)
    assert proof == oproof
    assert np.array_equal(cv, ocv)


@pytest.mark.parametrize("seed,widths,p_mul", [
    (301, [14, 6, 14], 0.6),   # wide input layer: almost every input row without mul gates
    (302, [12, 12, 12], 0.0),  # no mul gates: every phase-one hg row is copy-independent
    (303, [10, 13, 10], 1.0),  # every input row of the first layer with mul gates
    (304, [11, 9, 11, 9], 0.3),
])
def test_gpu_hg_rows_without_mul_gates(ctx, oracle, seed, widths, p_mul):
    """Phase-one hg rows whose input rows have no mul gates are left unwritten by rounds 1
    and 2 and recomputed from the add weights by rounds 2 and 3; mixes of such rows and
    gated rows must give the oracle's proof."""
    circ = gc.random_circuit(seed, widths, p_mul=p_mul, p_local=0.5, window=64)
    w = gc.random_witness(seed, circ.log_input_size, 16)
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


def test_pipelined_jobs_are_byte_identical(ctx):
    """Several proofs in flight (host stages overlapping device stages, mixed shapes and copy
    counts); each must still reproduce its reference golden, in any completion order."""
    names = ["cfg1_n16", "lanes1024", "mixed_widths_n16", "width_one_n8", "lanes48", "cfg1_n8"]
    built = [cases.build(n) for n in names]
    dcs = [ctx.load(c) for c, _, _ in built]
    jobs = []
    for (c, w, g), dc in zip(built, dcs):
        pb = np.empty(dc.proof_size(w.shape[1], g), np.uint8)
        cb = np.empty((3, w.shape[1]), np.uint32)
        jobs.append((ctx.submit(dc, w, pb, cb, grinding_bits=g), pb, cb))
    for name, (job, pb, cb) in zip(names, jobs):
        n = ctx.wait(job)
        assert sha(pb[:n].tobytes()) == GOLDEN[name]["proof_sha256"], name
        assert sha(cb.tobytes()) == GOLDEN[name]["claimed_v_sha256"], name


def test_failing_job_does_not_disturb_the_pipeline(ctx):
    from gkr_gb300._lib import GkrGpuError
    good = cases.build("cfg1_n16")
    bad_w = good[1].copy()
    bad_w[0, 0] = gc.P
    dc = ctx.load(good[0])
    bufs = [(np.empty(dc.proof_size(16), np.uint8), np.empty((3, 16), np.uint32)) for _ in range(3)]
    j0 = ctx.submit(dc, good[1], *bufs[0])
    j1 = ctx.submit(dc, bad_w, *bufs[1])
    j2 = ctx.submit(dc, good[1], *bufs[2])
    n0 = ctx.wait(j0)
    with pytest.raises(GkrGpuError):
        ctx.wait(j1)
    n2 = ctx.wait(j2)
    assert sha(bufs[0][0][:n0].tobytes()) == sha(bufs[2][0][:n2].tobytes()) == GOLDEN["cfg1_n16"]["proof_sha256"]


def test_device_input_pipeline(ctx):
    from gkr_gb300.prover import DeviceBuffer
    circ, w, g = cases.build("lanes256")
    dc = ctx.load(circ)
    d = DeviceBuffer(ctx, w.nbytes)
    d.upload(w)
    outs = [(np.empty(dc.proof_size(256), np.uint8), np.empty((3, 256), np.uint32)) for _ in range(2)]
    jobs = [ctx.submit(dc, None, pb, cb, d_input=d.ptr, marker=k) for k, (pb, cb) in enumerate(outs)]
    for job, (pb, cb) in zip(jobs, outs):
        n = ctx.wait(job)
        assert sha(pb[:n].tobytes()) == GOLDEN["lanes256"]["proof_sha256"]
    assert ctx.elapsed_ms(0, 1) >= 0.0


@pytest.mark.parametrize("seed,widths,n", [
    (401, [14, 10, 14, 9, 12], 32), (402, [16, 11, 15], 16), (403, [13, 8, 13, 6], 96), (404, [12, 9, 12], 1024),
    (405, [15, 12, 15], 160),
])
def test_gpu_sparse_layers_skip_groups_without_gates(ctx, oracle, seed, widths, n):
    """Layers much wider than their outputs: most pairs and quads of input rows are the first
    input of no gate, and most quads the second input of no mul gate.  Phase one's rounds 0
    and 1 and phase two's fused rounds 0 and 1 walk only the groups that have gates (their
    sums over the others are zero); the proof must be the oracle's."""
    circ = gc.random_circuit(seed, widths, p_mul=0.6, p_local=0.5, window=256)
    w = gc.random_witness(seed, circ.log_input_size, n)
    cv, proof = ctx.prove(ctx.load(circ), w)
    ocv, oproof = oracle.prove(circ, w)
    assert proof == oproof
    assert np.array_equal(cv, ocv)
