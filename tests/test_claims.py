"""The round claims the round kernels take p(1) from, checked on the oracle's proofs (CPU).

The GPU round kernels sum p(0) and p2raw only and write p(1) = claim - p(0).
- For phase one's round 0 the claim is alpha v(rz1) + beta v(rz2) per copy: the claimed
  values for the output layer, then the previous layer's vx and vy (sumcheck.hpp:129-132).
- For every later round of a phase it is the previous round's polynomial at its challenge
  (degree_2_eval, sumcheck_verifier_utils.hpp:10-18).

These tests replay the SHA-256 transcript over the proof bytes (transcript.hpp:87-175: a
challenge hashes the bytes appended since the previous one, or re-hashes the digest; its
value is the digest's first four bytes, little-endian, reduced mod p). They recover every
round polynomial and challenge, and check that p(0) + p(1) equals that claim in every such
round.  Phase two's round 0, whose claim also subtracts vx add(rz, rx) (sumcheck.hpp:158),
keeps its directly summed p(1) in the kernels and is not checked here.
"""
import hashlib

import numpy as np
import pytest

import cases

P = 2**31 - 1
INV2 = 1 << 30  # 2 * 2^30 = p + 1


def from_u32(x):
    s = (x & P) + (x >> 31)
    return s - P if s >= P else s


def degree2(v0, v1, v2, x):
    c2 = (INV2 * ((v2 - 2 * v1 + v0) % P)) % P
    c1 = (v1 - v0 - c2) % P
    return (v0 + ((c2 * x + c1) % P) * x) % P


class Replay:
    """Reads a proof front to back, keeping the transcript's hash state."""

    def __init__(self, proof):
        self.p = memoryview(proof)
        self.pos = 0
        self.start = 0  # first byte not yet hashed
        self.digest = bytes(32)

    def take(self, n):
        b = self.p[self.pos:self.pos + n]
        self.pos += n
        return b

    def row(self, n_copies):
        return np.frombuffer(self.take(4 * n_copies), np.uint32).astype(np.int64)

    def challenge(self):
        if self.pos > self.start:
            self.digest = hashlib.sha256(self.p[self.start:self.pos]).digest()
            self.start = self.pos
        else:
            self.digest = hashlib.sha256(self.digest).digest()
        return from_u32(int.from_bytes(self.digest[:4], "little"))


def check_claims(circ, n_copies, reps, claimed_v, proof):
    """Replays `proof` and returns the number of rounds whose claim was checked."""
    t = Replay(proof)
    t.take(4 * n_copies << circ.log_input_size)  # RAW commitment
    for _ in range(256 // 31):
        t.challenge()  # grinding's challenges (LinearGKR.hpp:13-32)
    t.take(32)
    for _ in range(circ.layers[-1].nb_output_vars):
        for _ in range(reps):
            t.challenge()  # rz1
    cv1 = [np.asarray(claimed_v[j], np.int64) for j in range(reps)]
    cv2 = [np.zeros(n_copies, np.int64) for _ in range(reps)]
    alpha, beta = 1, 0
    checked = 0
    for layer in reversed(circ.layers):
        n = layer.nb_input_vars
        claim = [(alpha * cv1[j] + beta * cv2[j]) % P for j in range(reps)]
        vx = [None] * reps
        for i_var in range(2 * n):
            for j in range(reps):
                p0, p1, p2 = t.row(n_copies), t.row(n_copies), t.row(n_copies)
                r = t.challenge()
                if i_var != n:  # not phase two's round 0
                    assert np.array_equal((p0 + p1) % P, claim[j]), (n, i_var, j)
                    checked += 1
                claim[j] = degree2(p0, p1, p2, r)
                if i_var == n - 1:
                    vx[j] = t.row(n_copies)
        vy = [t.row(n_copies) for _ in range(reps)]
        alpha, beta = t.challenge(), t.challenge()
        cv1, cv2 = vx, vy
    assert t.pos == len(proof)
    return checked


@pytest.mark.parametrize("name", ["cfg1_n16", "gkr_test_shape_n8", "mixed_widths_n16", "grind12_n16",
                                  "no_gates_rows_n16", "width_one_n8", "lanes48"])
def test_every_round_sums_to_its_claim(oracle, name):
    from oracle.oracle import num_repetitions
    circ, w, grind = cases.build(name)
    cv, proof = oracle.prove(circ, w, grinding_bits=grind)
    R = num_repetitions(grind)
    rounds = check_claims(circ, w.shape[1], R, cv, proof)
    assert rounds == R * sum(2 * l.nb_input_vars - 1 for l in circ.layers)


def test_a_wrong_p1_breaks_the_claim(oracle):
    """The replay is sensitive: changing one copy's p(1) in the second round of the top layer
    (its bytes re-hashed, so later challenges change too) fails the check at that round."""
    circ, w, grind = cases.build("cfg1_n16")
    cv, proof = oracle.prove(circ, w, grinding_bits=grind)
    N = w.shape[1]
    bad = bytearray(proof)
    at = (4 * N << circ.log_input_size) + 32 + 3 * (12 * N) + 4 * N  # round 1, rep 0, row p1, copy 0
    bad[at] ^= 1
    with pytest.raises(AssertionError):
        check_claims(circ, N, 3, cv, bytes(bad))
