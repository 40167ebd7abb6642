"""The algebra behind phase two's fused rounds 0 and 1 (k_p2_round01 + k_p2_round1_fin).

Round 1 folds the layer input v and the scalar table s at round 0's challenge r
(SumcheckMultiLinearProdHelper::receive_challenge, sumcheck_helper.hpp:104-133), so over
each group of four input rows its evaluations (poly_eval_at, sumcheck_helper.hpp:68-102)
are quadratic in r with coefficients that one pass over v can sum before r is known.  These
tests compute rounds 0 and 1 directly (fold, then sum) and from the nine per-group sums the
kernels keep, in exact integer arithmetic mod p, on random data and on edge values.
"""
import random

import pytest

P = 2**31 - 1


def fold(a, b, r):
    return (a + (b - a) * r) % P


def eval_at_two(p0, p1, p2raw):
    return (6 * p1 + 3 * p0 - 2 * p2raw) % P


def direct_round(f, h):
    """poly_eval_at over pairs (2i, 2i+1): (p(0), p(1), p(2))."""
    p0 = sum(f[2 * i] * h[2 * i] for i in range(len(f) // 2)) % P
    p1 = sum(f[2 * i + 1] * h[2 * i + 1] for i in range(len(f) // 2)) % P
    p2raw = sum((f[2 * i] + f[2 * i + 1]) * (h[2 * i] + h[2 * i + 1]) for i in range(len(f) // 2)) % P
    return p0, p1, eval_at_two(p0, p1, p2raw)


def sums(v, s):
    """The nine sums k_p2_round01 keeps per copy and repetition (E00, E11, QE, F22, F33, QF,
    U00, U11, QU) over groups of four rows; t0 = s0 + s2, t1 = s1 + s3 as k_s_build4 writes."""
    m = [0] * 9
    for g in range(len(v) // 4):
        x0, x1, x2, x3 = v[4 * g:4 * g + 4]
        s0, s1, s2, s3 = s[4 * g:4 * g + 4]
        u0, u1 = (x0 + x2) % P, (x1 + x3) % P
        t0, t1 = (s0 + s2) % P, (s1 + s3) % P
        terms = [x0 * s0, x1 * s1, (x0 + x1) % P * ((s0 + s1) % P), x2 * s2, x3 * s3,
                 (x2 + x3) % P * ((s2 + s3) % P), u0 * t0, u1 * t1, (u0 + u1) % P * ((t0 + t1) % P)]
        m = [(a + b) % P for a, b in zip(m, terms)]
    return m


def round0_from_sums(m):
    p0, p1, p2raw = (m[0] + m[3]) % P, (m[1] + m[4]) % P, (m[2] + m[5]) % P
    return p0, p1, eval_at_two(p0, p1, p2raw)


def round1_from_sums(m, r):
    m = list(m)
    for k in (2, 5, 8):  # cross sums from the pre-added products: K = Q - A - B
        m[k] = (m[k] - m[k - 2] - m[k - 1]) % P
    c0, c1, c2 = (1 - r) * (1 - r) % P, r * (1 - r) % P, r * r % P
    p0 = (c0 * m[0] + c1 * m[2] + c2 * m[1]) % P
    p1 = (c0 * m[3] + c1 * m[5] + c2 * m[4]) % P
    p2raw = (c0 * m[6] + c1 * m[8] + c2 * m[7]) % P
    return p0, p1, eval_at_two(p0, p1, p2raw)


def fold_table(t, r):
    return [fold(t[2 * i], t[2 * i + 1], r) for i in range(len(t) // 2)]


@pytest.mark.parametrize("rows,seed", [(4, 1), (8, 2), (64, 3), (256, 4)])
def test_rounds_0_and_1_from_the_nine_sums(rows, seed):
    rnd = random.Random(seed)
    v = [rnd.randrange(P) for _ in range(rows)]
    s = [rnd.randrange(P) for _ in range(rows)]
    r = rnd.randrange(P)
    m = sums(v, s)
    assert round0_from_sums(m) == direct_round(v, s)
    assert round1_from_sums(m, r) == direct_round(fold_table(v, r), fold_table(s, r))


@pytest.mark.parametrize("fill", [0, 1, P - 1])
def test_edge_values(fill):
    rnd = random.Random(fill)
    v = [fill] * 16
    s = [rnd.choice([0, 1, P - 1]) for _ in range(16)]
    for r in (0, 1, P - 1, 2):
        m = sums(v, s)
        assert round0_from_sums(m) == direct_round(v, s)
        assert round1_from_sums(m, r) == direct_round(fold_table(v, r), fold_table(s, r))


def test_round2_refold_equals_two_folds():
    """Round 2 refolds the layer input at both challenges instead of reading round 1's
    stored copies (k_p1_round2, k_p2_round2): the pairwise fold twice is that table."""
    rnd = random.Random(9)
    v = [rnd.randrange(P) for _ in range(64)]
    r0, r1 = rnd.randrange(P), rnd.randrange(P)
    stored = fold_table(fold_table(v, r0), r1)
    refold = [fold(fold(v[4 * q], v[4 * q + 1], r0), fold(v[4 * q + 2], v[4 * q + 3], r0), r1) for q in range(16)]
    assert stored == refold
