"""Host logic of the serving loop (no GPU): the device arena that holds resident witnesses
hands out aligned, disjoint ranges, merges freed neighbours and refuses what does not fit."""
import numpy as np

from gkr_gb300.serving import ALIGN, Arena


def test_alloc_aligned_disjoint_and_full():
    a = Arena(10 * ALIGN)
    offs = [a.alloc(n) for n in (1, ALIGN, ALIGN + 1, 3 * ALIGN)]
    assert offs == [0, ALIGN, 2 * ALIGN, 4 * ALIGN]
    assert all(o % ALIGN == 0 for o in offs)
    assert a.in_use() == 7 * ALIGN
    assert a.alloc(4 * ALIGN) is None  # 3 blocks left
    assert a.alloc(3 * ALIGN) == 7 * ALIGN
    assert a.alloc(1) is None


def test_release_merges_neighbours():
    a = Arena(8 * ALIGN)
    x, y, z = a.alloc(2 * ALIGN), a.alloc(2 * ALIGN), a.alloc(2 * ALIGN)
    a.release(x)
    a.release(z)
    assert a.alloc(5 * ALIGN) is None  # free: [0, 2) and [4, 8) blocks, not contiguous
    a.release(y)
    assert a.free == [(0, 8 * ALIGN)]
    assert a.alloc(8 * ALIGN) == 0


def test_random_sequence_never_overlaps():
    rng = np.random.default_rng(5)
    a = Arena(1 << 20)
    live = {}
    for _ in range(2000):
        if live and rng.random() < 0.45:
            off = list(live)[rng.integers(len(live))]
            a.release(off)
            del live[off]
        else:
            n = int(rng.integers(1, 1 << 15))
            off = a.alloc(n)
            if off is not None:
                live[off] = -(-n // ALIGN) * ALIGN
        spans = sorted(live.items())
        for (o1, n1), (o2, _) in zip(spans, spans[1:]):
            assert o1 + n1 <= o2
        assert all(o + n <= a.size for o, n in spans)
        assert a.in_use() == sum(live.values())
