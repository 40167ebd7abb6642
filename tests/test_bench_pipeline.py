"""Host logic of bench.py's pipelined timing (no GPU): the timed region runs from the
earliest device-stage beginning among the timed proofs to the latest device-stage end among
them, so a proof whose device work mostly lay before the region cannot be counted inside it;
with several device lanes proofs can finish out of order; at most `depth` proofs are in
flight, and the kernel statistics bracket the timed proofs."""
import pytest

import bench


class FakeCtx:
    """Proof i's device stage runs from begins[i] to ends[i] ms after the reference mark.
    A proof submitted with marker k records its end in slot k and its beginning in slot
    64 + k; gkrgpu_mark records the reference slot at time 0."""

    def __init__(self, begins, ends):
        self.begins, self.ends = begins, ends
        self.marker_ms = {}
        self.waited = []
        self.in_flight = 0
        self.max_in_flight = 0
        self.next_id = 0

    def mark(self, slot):
        assert self.in_flight == 0, "the reference mark is taken before any proof is submitted"
        self.marker_ms[slot] = 0.0

    def submit(self, buf, marker):
        i = self.next_id
        self.next_id += 1
        self.in_flight += 1
        self.max_in_flight = max(self.max_in_flight, self.in_flight)
        if marker >= 0:
            self.marker_ms[marker] = self.ends[i]
            self.marker_ms[64 + marker] = self.begins[i]
        return i

    def wait(self, job):
        self.in_flight -= 1
        self.waited.append(job)

    def kernel_stats(self):
        return {"k": {"launches": len(self.waited), "ms": 0.0, "bytes": 0.0}}

    def elapsed_ms(self, a, b):
        return self.marker_ms[b] - self.marker_ms[a]


def run(begins, ends, n_warm, n_timed, depth):
    ctx = FakeCtx(begins, ends)
    bufs = [None] * depth
    out = bench.pipelined(ctx, n_warm, n_timed, bufs, lambda b, m: ctx.submit(b, m))
    return ctx, out


def test_region_starts_at_the_first_timed_device_stage_and_ends_at_the_last_end():
    # two lanes: warm-up proofs 0-2, timed 3-5; proof 3 began at 9.5 (while warm-up proof 2
    # was still running) and ended at 20.5, just after proof 2; proof 4 (timed) ends after
    # proof 5, the last one submitted
    begins = [0.0, 0.0, 10.0, 9.5, 20.5, 21.0]
    ends = [10.0, 9.5, 20.0, 20.5, 32.0, 30.0]
    ctx, (total, steps, lat, s0, s1, stage) = run(begins, ends, n_warm=3, n_timed=3, depth=4)
    # from proof 3's beginning, not from the end of the last warm-up proof (20.0), which would
    # count proof 3's 11 ms of device work inside a 12 ms window
    assert total == 32.0 - 9.5
    assert steps == [20.5 - 9.5, 30.0 - 20.5, 32.0 - 30.0]
    assert stage == [11.0, 11.5, 9.0]
    assert len(lat) == 3
    assert ctx.max_in_flight <= 4
    assert s0["k"]["launches"] == 3 and s1["k"]["launches"] == 6


def test_in_order_region_and_depth_bound():
    ends = [float(10 * (i + 1)) for i in range(8)]
    begins = [e - 10.0 for e in ends]
    ctx, (total, steps, _, _, _, _) = run(begins, ends, n_warm=3, n_timed=5, depth=2)
    assert total == 80.0 - 30.0
    assert steps == [10.0] * 5
    assert ctx.max_in_flight <= 2
    assert ctx.waited == list(range(8))


def test_timed_proofs_fit_the_marker_slots():
    with pytest.raises(ValueError):
        bench.pipelined(FakeCtx([0.0] * 70, [1.0] * 70), 1, bench.MAX_TIMED + 1, [None], lambda b, m: 0)


def test_a_failed_proof_drains_the_others_before_unwinding():
    class Failing(FakeCtx):
        def wait(self, job):
            super().wait(job)
            if job == 2:
                raise RuntimeError("proof 2 failed")

    ctx = Failing([0.0] * 8, [float(i + 1) for i in range(8)])
    with pytest.raises(RuntimeError):
        bench.pipelined(ctx, 2, 6, [None] * 4, lambda b, m: ctx.submit(b, m))
    # proofs 0..5 were submitted (depth 4 after two waits); every one of them was waited for
    assert sorted(ctx.waited) == list(range(ctx.next_id))
    assert ctx.in_flight == 0


def test_reference_formula_bytes_by_hand():
    """One layer, 4 inputs, 2 outputs, one mul and one add gate, 4 copies of M31, R = 3:
    (2 + 1 + 2) + (1 + 12) + 16 * 4 + 7 * 4 = 110 vectors, plus the 2 output rows, of 16
    bytes, and 48 + 24 + 12 * (4 + 8) bytes of gate lists and scalar tables."""
    import numpy as np
    from gkr_gb300 import circuit as gc
    layer = gc.CircuitLayer(1, 2, mul=np.array([[0, 1, 2, 1]], np.uint32), add=np.array([[1, 3, 1]], np.uint32))
    circ = gc.Circuit([layer])
    assert bench.reference_formula_bytes(circ, 4) == 112 * 16 + 48 + 24 + 12 * 12
