"""Host logic of the serving loop (no GPU): the device arena that holds resident witnesses
hands out aligned, disjoint ranges, merges freed neighbours and refuses what does not fit;
the proof-buffer pool reuses buffers across sizes of one class and keeps to its cap."""
import numpy as np

from gkr_gb300.serving import ALIGN, Arena, BufferPool


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


def test_buffer_pool_classes_and_cap():
    assert BufferPool.size_class(1) == 1 << 20
    assert BufferPool.size_class((1 << 20) + 1) == 1 << 21
    assert BufferPool.size_class(3 << 20) == 4 << 20
    pool = BufferPool(8 << 20)
    assert pool.take(3 << 20) is None
    a = np.empty(BufferPool.size_class(3 << 20), np.uint8)
    assert pool.give(a)
    assert pool.take((2 << 20) + 1) is a  # another size of the same class
    assert pool.take(3 << 20) is None
    b, c = np.empty(4 << 20, np.uint8), np.empty(4 << 20, np.uint8)
    assert pool.give(b) and pool.give(c)
    assert not pool.give(np.empty(1 << 20, np.uint8))  # over the cap
    assert not pool.give(np.empty(3 << 20, np.uint8))  # not a class size
    assert pool.pooled == 8 << 20
    assert pool.take(4 << 20) is not None and pool.pooled == 4 << 20
