"""Proof files in the reference's format (Proof::write_and_compress / read_proof,
include/fiat_shamir/transcript.hpp:54-84): a 4-byte little-endian length, then the bytes.
Host-only entry points of the C ABI (gkrgpu_proof_write / gkrgpu_proof_read)."""
import ctypes
import struct

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    from gkr_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.mark.parametrize("n", [0, 1, 31, 4096, 80416])
def test_round_trip_and_byte_format(tmp_path, lib, n):
    from gkr_gb300.prover import Proof
    data = np.random.default_rng(n).integers(0, 256, n, dtype=np.uint8).tobytes()
    path = tmp_path / "proof.txt"
    Proof(data).write(path)
    raw = path.read_bytes()
    # the file the reference writes: uint32 length (little-endian on x86-64 and aarch64), then the bytes
    assert raw == struct.pack("<I", n) + data
    assert Proof.read(path) == Proof(data)


def test_reads_a_file_written_in_the_reference_layout(tmp_path, lib):
    from gkr_gb300.prover import Proof
    body = bytes(range(200)) * 3
    path = tmp_path / "ref_proof.txt"
    path.write_bytes(struct.pack("<I", len(body)) + body)
    assert Proof.read(path).bytes == body


def test_errors(tmp_path, lib):
    from gkr_gb300 import _lib
    n = ctypes.c_uint64()
    assert lib.gkrgpu_proof_read(str(tmp_path / "missing").encode(), None, 0, ctypes.byref(n)) == _lib.ERR_IO
    short = tmp_path / "short.txt"
    short.write_bytes(struct.pack("<I", 100) + b"x" * 10)
    buf = np.empty(100, np.uint8)
    assert lib.gkrgpu_proof_read(str(short).encode(), buf.ctypes.data, 100, ctypes.byref(n)) == _lib.ERR_IO
    assert lib.gkrgpu_proof_read(str(short).encode(), buf.ctypes.data, 50, ctypes.byref(n)) == _lib.ERR_CAPACITY
    assert n.value == 100
    assert lib.gkrgpu_proof_read(str(short).encode(), None, 0, ctypes.byref(n)) == _lib.OK and n.value == 100
    stub = tmp_path / "stub.txt"
    stub.write_bytes(b"\x01\x00")
    assert lib.gkrgpu_proof_read(str(stub).encode(), None, 0, ctypes.byref(n)) == _lib.ERR_IO
    # a length that does not fit the 32-bit field is refused (nothing is read from the pointer)
    assert lib.gkrgpu_proof_write(str(tmp_path / "big").encode(), buf.ctypes.data, 1 << 32) == _lib.ERR_INVALID
