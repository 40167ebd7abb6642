"""GPU tests of the persistent phase tails: a phase's last rounds, on small tables, run in
one launch that waits on the device (bounded) for each round's challenges, which the host
writes to host-mapped memory.  Proofs must be byte-identical with the tails on and off and
equal the oracle's (exact arithmetic: tolerance zero), for copy counts whose tiles leave
threads idle (28: 7 threads per row slice) and for layers whose whole phase is one tail.
The bounded wait is made to expire on purpose (a challenge that never comes): the kernel
must return, report it, and leave the context usable."""
import numpy as np
import pytest

from gkr_gb300 import circuit as gc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,widths,n", [
    (501, [9, 10, 9, 11, 8], 16), (502, [12, 8, 12], 1024), (503, [7, 9, 7], 28), (504, [6, 6, 6, 6], 4),
    (505, [11, 10, 11], 96), (506, [13, 12], 160), (507, [5, 10, 5], 256),
])
def test_tails_on_and_off_give_the_oracle_proof(ctx, oracle, seed, widths, n):
    circ = gc.random_circuit(seed, widths, p_mul=0.6, p_local=0.7, window=64)
    w = gc.random_witness(seed, circ.log_input_size, n)
    dc = ctx.load(circ)
    try:
        ctx.set_round_tail(False)
        cv0, p0 = ctx.prove(dc, w)
    finally:
        ctx.set_round_tail(True)
    cv1, p1 = ctx.prove(dc, w)
    assert p1 == p0
    assert np.array_equal(cv1, cv0)
    ocv, op = oracle.prove(circ, w)
    assert p1 == op and np.array_equal(cv1, ocv)


def test_tails_in_concurrent_lanes(oracle):
    from gkr_gb300 import build as libbuild
    libbuild.build()
    from gkr_gb300.prover import Context
    c = Context(0)
    try:
        c.set_concurrency(lanes=4)
        # proofs of 2^8 .. 2^14-row layers in four lanes at once, each with its own tails
        specs = [(511 + i, [8 + i % 3, 9, 8 + i % 2], 16 * (1 + i % 4)) for i in range(8)]
        specs += [(531, [13, 12, 13], 16), (532, [14, 13], 32), (533, [12, 14, 12], 64), (534, [14, 11, 14], 16)]
        circs = [gc.random_circuit(s, wd) for s, wd, _ in specs]
        wits = [gc.random_witness(s, cc.log_input_size, n) for (s, _, n), cc in zip(specs, circs)]
        dcs = [c.load(cc) for cc in circs]
        bufs = [(np.empty(d.proof_size(w.shape[1]), np.uint8), np.empty((3, w.shape[1]), np.uint32))
                for d, w in zip(dcs, wits)]
        jobs = [c.submit(d, w, b[0], b[1]) for d, w, b in zip(dcs, wits, bufs)]
        lens = [c.wait(j) for j in jobs]
        for cc, w, b, ln in zip(circs, wits, bufs, lens):
            ocv, op = oracle.prove(cc, w)
            assert b[0][:ln].tobytes() == op
    finally:
        c.close()


def test_bounded_wait_expires_and_the_context_stays_usable(ctx, oracle):
    expired, published = ctx.check_device_wait(2000)
    assert expired and published == 1
    circ = gc.random_circuit(520, [7, 8, 7])
    w = gc.random_witness(520, circ.log_input_size, 16)
    cv, proof = ctx.prove(ctx.load(circ), w)
    assert proof == oracle.prove(circ, w)[1]
