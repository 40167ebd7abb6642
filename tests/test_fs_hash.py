"""The Keccak-256 transcript option (FiatShamir_hash_type::Keccak256,
include/configuration/config.hpp:18-24), on the CPU.

The reference names Keccak256 but its transcript only implements SHA-256, so there is no
reference output to pin this mode to: the sponge is checked against known answers and
against Python's SHA3-256 (the same permutation with the FIPS 202 domain byte), and the
transcript against the oracle's own prover/verifier round trip.  The product's Keccak
(expander-cpp_gb300/csrc/keccak.cpp) and the oracle's (oracle/fs_hash.c) are written
independently."""
import hashlib

import pytest

import cases

KECCAK_EMPTY = "c5d2460186f7233c927e7db2dcc703c0e500b653ca82273b7bfad8045d85a470"
KECCAK_ABC = "4e03657aea45a94fc7d47ba826c8d667c0d1e6e33a64a036ec44f58fa12d6c45"
# block-boundary lengths of the 136-byte rate, and several blocks
LENGTHS = [0, 1, 3, 31, 32, 64, 135, 136, 137, 271, 272, 273, 1000, 4096]


def _data(n):
    return bytes((i * 131 + 7) & 0xFF for i in range(n))


@pytest.fixture(scope="module")
def lib():
    from gkr_gb300 import _lib, build
    build.build()
    return _lib


def test_oracle_keccak_known_answers(oracle):
    assert oracle.keccak256(b"").hex() == KECCAK_EMPTY
    assert oracle.keccak256(b"abc").hex() == KECCAK_ABC


@pytest.mark.parametrize("n", LENGTHS)
def test_oracle_sponge_matches_sha3(oracle, n):
    d = _data(n)
    assert oracle.sha3_256(d) == hashlib.sha3_256(d).digest()


def test_product_keccak_known_answers(lib):
    assert lib.keccak256(b"").hex() == KECCAK_EMPTY
    assert lib.keccak256(b"abc").hex() == KECCAK_ABC


@pytest.mark.parametrize("n", LENGTHS)
def test_product_sponge_matches_sha3_and_oracle(lib, oracle, n):
    d = _data(n)
    assert lib.sha3_256(d) == hashlib.sha3_256(d).digest()
    assert lib.keccak256(d) == oracle.keccak256(d)


def test_config_accepts_only_known_hashes():
    from gkr_gb300.prover import Config
    assert Config().FS_hash == "SHA256"
    assert Config(FS_hash="Keccak256").FS_hash == "Keccak256"
    with pytest.raises(ValueError):
        Config(FS_hash="Poseidon")


def test_set_fs_hash_rejects_null_context(lib):
    L = lib.load()
    assert L.gkrgpu_set_fs_hash(None, 1) != 0
    assert L.gkrgpu_last_error()


@pytest.mark.parametrize("name", ["cfg1_n16", "mixed_widths_n16", "grind8_n16"])
def test_oracle_keccak_transcript_round_trip(oracle, name):
    circ, w, g = cases.build(name)
    sha_cv, sha_proof = oracle.prove(circ, w, grinding_bits=g)
    try:
        oracle.set_fs_hash("Keccak256")
        cv, proof = oracle.prove(circ, w, grinding_bits=g)
        assert len(proof) == len(sha_proof)
        assert proof != sha_proof
        # the commitment (input rows) is the same; the challenges after it are not
        com = (1 << circ.log_input_size) * w.shape[1] * 4
        assert proof[:com] == sha_proof[:com]
        assert oracle.verify(circ, w, cv, proof, grinding_bits=g)
        assert not oracle.verify(circ, w, sha_cv, sha_proof, grinding_bits=g)
        bad = bytearray(proof)
        bad[len(bad) // 2] ^= 1
        assert not oracle.verify(circ, w, cv, bytes(bad), grinding_bits=g)
    finally:
        oracle.set_fs_hash("SHA256")
    assert not oracle.verify(circ, w, cv, proof, grinding_bits=g)
    assert oracle.verify(circ, w, sha_cv, sha_proof, grinding_bits=g)


@pytest.mark.parametrize("name", ["bn_mixed_widths_n16", "bn_grind0_n8"])
def test_oracle_bn254_keccak_transcript_round_trip(name):
    from oracle.oracle import OracleBn254
    obn = OracleBn254()
    circ, w, g = cases.build_bn(name)
    sha_cv, sha_proof = obn.prove(circ, w, grinding_bits=g)
    try:
        obn.set_fs_hash("Keccak256")
        cv, proof = obn.prove(circ, w, grinding_bits=g)
        assert len(proof) == len(sha_proof) and proof != sha_proof
        assert obn.verify(circ, w, cv, proof, grinding_bits=g)
        assert not obn.verify(circ, w, sha_cv, sha_proof, grinding_bits=g)
    finally:
        obn.set_fs_hash("SHA256")
    assert not obn.verify(circ, w, cv, proof, grinding_bits=g)
