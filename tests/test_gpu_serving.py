"""GPU tests of the serving loop (gkr_gb300.serving.ProofServer): requests of mixed sizes
arriving together are admitted, their witnesses uploaded once into the resident arena, and
proved with overlapping device stages; every request's proof and claims must be the same as
the same proof made alone, with nothing else running (exact: tolerance zero).  Also: a
request that arrives when the server is idle, and admission control."""
import numpy as np
import pytest

from gkr_gb300 import circuit as gc

pytestmark = pytest.mark.gpu

# (seed, depth, width, copies): mixed-workload shapes, small enough for the test
SPECS = [(41, 4, 10, 16), (42, 6, 12, 64), (43, 3, 8, 32), (44, 5, 14, 16), (45, 4, 11, 128), (46, 7, 9, 48),
         (47, 4, 13, 32), (48, 3, 12, 256), (49, 6, 10, 16), (50, 4, 8, 64)]


@pytest.fixture(scope="module")
def jobs():
    from gkr_gb300 import build as libbuild
    libbuild.build()
    from gkr_gb300.prover import Context
    ctx = Context(0)
    circs = [gc.uniform_circuit(s, d, k) for s, d, k, _ in SPECS]
    wits = [gc.random_witness(s, k, n) for s, _, k, n in SPECS]
    dcs = [ctx.load(c) for c in circs]
    alone = [ctx.prove(dc, w) for dc, w in zip(dcs, wits)]  # one at a time, nothing else running
    yield ctx, dcs, wits, alone
    ctx.close()


def test_requests_in_the_mix_equal_the_proofs_made_alone(jobs):
    from gkr_gb300.serving import ProofServer
    ctx, dcs, wits, alone = jobs
    srv = ProofServer(ctx, lanes=4, budget_bytes=8 << 30, arena_bytes=1 << 30)
    try:
        futs = [srv.submit(dc, w) for dc, w in zip(dcs, wits)]
        futs += [srv.submit(dcs[i], wits[i]) for i in (3, 1, 4)]  # repeats while the first ones run
        res = [f.result(timeout=120) for f in futs]
    finally:
        srv.close()
    for i, r in enumerate(res[:len(SPECS)]):
        cv, proof = alone[i]
        assert r.proof.tobytes() == proof, i
        assert np.array_equal(r.claimed_v, cv), i
        assert r.latency_ms >= r.admit_wait_ms >= 0
    for i, r in zip((3, 1, 4), res[len(SPECS):]):
        assert r.proof.tobytes() == alone[i][1]
    st = srv.stats()
    assert st["admitted"] == len(futs) and st["rejected"] == 0 and st["completed"] == len(futs)
    assert 0 < st["witness_peak_bytes"] <= st["arena_bytes"]
    assert 0 < st["workspace_peak_bytes"] <= st["budget_bytes"]


def test_released_proof_buffers_are_reused(jobs):
    from gkr_gb300.serving import ProofServer
    ctx, dcs, wits, alone = jobs
    srv = ProofServer(ctx, lanes=2, budget_bytes=4 << 30, arena_bytes=256 << 20)
    try:
        first = srv.submit(dcs[2], wits[2]).result(timeout=60)
        assert first.proof.tobytes() == alone[2][1]
        buf = first._buf
        first.release()
        again = srv.submit(dcs[2], wits[2]).result(timeout=60)
        assert again._buf is buf  # the same memory, rewritten
        assert again.proof.tobytes() == alone[2][1]
        other = srv.submit(dcs[5], wits[5]).result(timeout=60)  # `again` still holds buf
        assert other.proof.tobytes() == alone[5][1]
        assert other._buf is not buf
    finally:
        srv.close()


def test_request_on_an_idle_server(jobs):
    from gkr_gb300.serving import ProofServer
    ctx, dcs, wits, alone = jobs
    srv = ProofServer(ctx, lanes=2, budget_bytes=4 << 30, arena_bytes=256 << 20)
    try:
        r = srv.submit(dcs[1], wits[1]).result(timeout=60)
    finally:
        srv.close()
    assert r.proof.tobytes() == alone[1][1]


def test_admission_queue_rejects_beyond_its_bound(jobs):
    from gkr_gb300.serving import ProofServer, Rejected
    ctx, dcs, wits, alone = jobs
    # one request in flight at a time, and at most two waiting for admission
    srv = ProofServer(ctx, lanes=1, arena_bytes=256 << 20, max_queue=2, max_admitted=1)
    try:
        futs = [srv.submit(dcs[i], wits[i]) for i in range(8)]
        out = []
        for i, f in enumerate(futs):
            try:
                out.append((i, f.result(timeout=60)))
            except Rejected:
                out.append((i, None))
    finally:
        srv.close()
    done = [(i, r) for i, r in out if r is not None]
    assert srv.stats()["rejected"] == 8 - len(done) > 0
    for i, r in done:
        assert r.proof.tobytes() == alone[i][1]
