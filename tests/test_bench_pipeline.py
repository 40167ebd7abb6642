"""Host logic of bench.py's pipelined timing (no GPU): with several device lanes proofs can
finish out of order, and the timed region must still end only when every timed proof has
finished; at most `depth` proofs are in flight, and the kernel statistics bracket the
timed proofs."""
import bench


class FakeCtx:
    """Proof i ends at `ends[i]` ms; a marker records the end of the proof submitted with it."""

    def __init__(self, ends):
        self.ends = ends
        self.marker_ms = {}
        self.waited = []
        self.in_flight = 0
        self.max_in_flight = 0
        self.next_id = 0

    def submit(self, buf, marker):
        i = self.next_id
        self.next_id += 1
        self.in_flight += 1
        self.max_in_flight = max(self.max_in_flight, self.in_flight)
        if marker >= 0:
            self.marker_ms[marker] = self.ends[i]
        return i

    def wait(self, job):
        self.in_flight -= 1
        self.waited.append(job)

    def kernel_stats(self):
        return {"k": {"launches": len(self.waited), "ms": 0.0, "bytes": 0.0}}

    def elapsed_ms(self, a, b):
        return self.marker_ms[b] - self.marker_ms[a]


def run(ends, n_warm, n_timed, depth):
    ctx = FakeCtx(ends)
    bufs = [None] * depth
    out = bench.pipelined(ctx, n_warm, n_timed, bufs, lambda b, m: ctx.submit(b, m))
    return ctx, out


def test_region_ends_at_the_last_timed_proof_even_out_of_order():
    # two lanes: proof 4 (timed) finishes after proof 5 (the last submitted)
    ends = [10.0, 11.0, 20.0, 21.0, 32.0, 30.0]
    ctx, (total, steps, lat, s0, s1) = run(ends, n_warm=3, n_timed=3, depth=4)
    # from the last warm-up proof's end (proof 2) to the latest timed end (proof 4), not to
    # the end of the last submitted proof (proof 5, 30 ms)
    assert total == 32.0 - 20.0
    assert len(steps) == 3 and len(lat) == 3
    assert ctx.max_in_flight <= 4
    assert s0["k"]["launches"] == 3 and s1["k"]["launches"] == 6


def test_in_order_region_and_depth_bound():
    ends = [float(10 * i) for i in range(8)]
    ctx, (total, steps, _, _, _) = run(ends, n_warm=3, n_timed=5, depth=2)
    assert total == 70.0 - 20.0
    assert steps == [10.0] * 5
    assert ctx.max_in_flight <= 2
    assert ctx.waited == list(range(8))
