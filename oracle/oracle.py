"""Test infrastructure only: ctypes bindings to the CPU oracle.

``Oracle`` wraps the C restatement (oracle/build/libgkr_oracle.so); ``Reference``
wraps the compiled reference driver (oracle/_ref/libgkr_ref.so), present only where the
reference tree was available at build time.  Circuits are gkr_gb300.circuit.Circuit
objects (any object with .layers of nb_output_vars / nb_input_vars / mul / add).
"""
import ctypes
import os

import numpy as np

from . import build as _build


class _Layer(ctypes.Structure):
    _fields_ = [("nb_output_vars", ctypes.c_uint32), ("nb_input_vars", ctypes.c_uint32),
                ("n_mul", ctypes.c_uint64), ("n_add", ctypes.c_uint64),
                ("mul", ctypes.c_void_p), ("add", ctypes.c_void_p)]


def _layers(circuit):
    keep = []
    arr = (_Layer * len(circuit.layers))()
    for k, l in enumerate(circuit.layers):
        m = np.ascontiguousarray(l.mul, dtype=np.uint32)
        a = np.ascontiguousarray(l.add, dtype=np.uint32)
        keep += [m, a]
        arr[k] = _Layer(l.nb_output_vars, l.nb_input_vars, m.shape[0], a.shape[0],
                        m.ctypes.data if m.size else None, a.ctypes.data if a.size else None)
    return arr, keep


def num_repetitions(grinding_bits=10):
    s = 100 - grinding_bits
    return s // 31 + (s % 31 != 0)


def proof_size(circuit, n_copies, reps):
    rows = sum(reps * (6 * l.nb_input_vars + 2) for l in circuit.layers)
    return (1 << circuit.layers[0].nb_input_vars) * n_copies * 4 + 32 + rows * n_copies * 4


FS_HASHES = {"SHA256": 0, "Keccak256": 1}


class _FsHash:
    """Transcript-hash selection and the Keccak sponge of oracle/fs_hash.c (process-wide)."""

    def set_fs_hash(self, name: str):
        self.lib.oracle_set_fs_hash.argtypes = [ctypes.c_int]
        self.lib.oracle_set_fs_hash(FS_HASHES[name])

    def _digest(self, fn, data):
        b = np.frombuffer(bytes(data), np.uint8)
        out = np.empty(32, np.uint8)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
        fn(b.ctypes.data if len(b) else None, len(b), out.ctypes.data)
        return out.tobytes()

    def keccak256(self, data: bytes) -> bytes:
        return self._digest(self.lib.oracle_keccak256, data)

    def sha3_256(self, data: bytes) -> bytes:
        return self._digest(self.lib.oracle_sha3_256, data)


class Oracle(_FsHash):
    """The C restatement of the reference prover/verifier."""

    def __init__(self, path=None):
        path = path or _build.build_oracle()
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.oracle_prove.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), ctypes.c_void_p]
        L.oracle_verify.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
        L.oracle_evaluate.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_eval_multilinear.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p,
                                              ctypes.c_void_p]
        L.oracle_sha256.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
        L.oracle_bench.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int]
        L.oracle_bench.restype = ctypes.c_double

    def prove(self, circuit, witness, grinding_bits=10):
        """Returns (claimed_v (R, N) uint32, proof bytes)."""
        w = np.ascontiguousarray(witness, dtype=np.uint32)
        N = w.shape[1]
        R = num_repetitions(grinding_bits)
        cap = proof_size(circuit, N, R)
        proof = np.empty(cap, np.uint8)
        cv = np.empty((R, N), np.uint32)
        plen = ctypes.c_uint64()
        arr, keep = _layers(circuit)
        rc = self.lib.oracle_prove(arr, len(circuit.layers), N, w.ctypes.data, grinding_bits, proof.ctypes.data, cap,
                                   ctypes.byref(plen), cv.ctypes.data)
        if rc != 0:
            raise ValueError(f"oracle_prove failed rc={rc}")
        return cv, proof[:plen.value].tobytes()

    def verify(self, circuit, witness, claimed_v, proof, grinding_bits=10):
        w = np.ascontiguousarray(witness, dtype=np.uint32)
        cv = np.ascontiguousarray(claimed_v, dtype=np.uint32)
        pb = np.frombuffer(bytes(proof), np.uint8)
        arr, keep = _layers(circuit)
        rc = self.lib.oracle_verify(arr, len(circuit.layers), w.shape[1], w.ctypes.data, grinding_bits,
                                    pb.ctypes.data, len(pb), cv.ctypes.data)
        if rc < 0:
            raise ValueError("oracle_verify: bad input")
        return rc == 1

    def evaluate(self, circuit, witness):
        """Every layer's input rows then the last layer's output rows, as a list of arrays."""
        w = np.ascontiguousarray(witness, dtype=np.uint32)
        N = w.shape[1]
        sizes = [1 << l.nb_input_vars for l in circuit.layers] + [1 << circuit.layers[-1].nb_output_vars]
        out = np.empty((sum(sizes), N), np.uint32)
        arr, keep = _layers(circuit)
        if self.lib.oracle_evaluate(arr, len(circuit.layers), N, w.ctypes.data, out.ctypes.data) != 0:
            raise ValueError("oracle_evaluate: bad input")
        return np.split(out, np.cumsum(sizes)[:-1])

    def eval_multilinear(self, evals, r):
        e = np.ascontiguousarray(evals, dtype=np.uint32)
        rr = np.ascontiguousarray(r, dtype=np.uint32)
        out = np.empty(e.shape[1], np.uint32)
        self.lib.oracle_eval_multilinear(e.ctypes.data, len(rr), e.shape[1], rr.ctypes.data, out.ctypes.data)
        return out

    def sha256(self, data: bytes) -> bytes:
        b = np.frombuffer(bytes(data), np.uint8)
        out = np.empty(32, np.uint8)
        self.lib.oracle_sha256(b.ctypes.data if len(b) else None, len(b), out.ctypes.data)
        return out.tobytes()

    def bench(self, circuit, witness, n_threads, proofs_per_thread, grinding_bits=10):
        """Wall seconds for n_threads x proofs_per_thread proofs (evaluate + prove)."""
        w = np.ascontiguousarray(witness, dtype=np.uint32)
        arr, keep = _layers(circuit)
        t = self.lib.oracle_bench(arr, len(circuit.layers), w.shape[1], w.ctypes.data, grinding_bits, n_threads,
                                  proofs_per_thread)
        if t < 0:
            raise RuntimeError("oracle_bench failed")
        return t


class OracleBn254(_FsHash):
    """The C restatement over BN254 (oracle/gkr_oracle_bn254.c).  Tables are (rows, N, 4)
    uint64 limb arrays; claimed_v is (1, N, 4)."""

    def __init__(self, path=None):
        path = path or _build.build_oracle()
        self.lib = ctypes.CDLL(path)
        L = self.lib
        P, I, U32, U64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64
        L.oracle_bn254_prove.argtypes = [P, I, U32, P, I, P, U64, ctypes.POINTER(U64), P]
        L.oracle_bn254_verify.argtypes = [P, I, U32, P, I, P, U64, P]
        L.oracle_bn254_evaluate.argtypes = [P, I, U32, P, P]
        L.oracle_bn254_proof_size.argtypes = [P, I, U32]
        L.oracle_bn254_proof_size.restype = U64
        L.oracle_bn254_bench.argtypes = [P, I, U32, P, I, I, I]
        L.oracle_bn254_bench.restype = ctypes.c_double

    def proof_size(self, circuit, n_copies):
        arr, keep = _layers(circuit)
        return self.lib.oracle_bn254_proof_size(arr, len(circuit.layers), n_copies)

    def prove(self, circuit, witness, grinding_bits=10):
        w = np.ascontiguousarray(witness, dtype=np.uint64)
        N = w.shape[1]
        cap = self.proof_size(circuit, N)
        proof = np.empty(cap, np.uint8)
        cv = np.empty((1, N, 4), np.uint64)
        plen = ctypes.c_uint64()
        arr, keep = _layers(circuit)
        rc = self.lib.oracle_bn254_prove(arr, len(circuit.layers), N, w.ctypes.data, grinding_bits, proof.ctypes.data,
                                         cap, ctypes.byref(plen), cv.ctypes.data)
        if rc != 0:
            raise ValueError(f"oracle_bn254_prove failed rc={rc}")
        return cv, proof[:plen.value].tobytes()

    def verify(self, circuit, witness, claimed_v, proof, grinding_bits=10):
        w = np.ascontiguousarray(witness, dtype=np.uint64)
        cv = np.ascontiguousarray(claimed_v, dtype=np.uint64)
        pb = np.frombuffer(bytes(proof), np.uint8)
        arr, keep = _layers(circuit)
        rc = self.lib.oracle_bn254_verify(arr, len(circuit.layers), w.shape[1], w.ctypes.data, grinding_bits,
                                          pb.ctypes.data, len(pb), cv.ctypes.data)
        if rc < 0:
            raise ValueError("oracle_bn254_verify: bad input")
        return rc == 1

    def evaluate(self, circuit, witness):
        w = np.ascontiguousarray(witness, dtype=np.uint64)
        N = w.shape[1]
        sizes = [1 << l.nb_input_vars for l in circuit.layers] + [1 << circuit.layers[-1].nb_output_vars]
        out = np.empty((sum(sizes), N, 4), np.uint64)
        arr, keep = _layers(circuit)
        if self.lib.oracle_bn254_evaluate(arr, len(circuit.layers), N, w.ctypes.data, out.ctypes.data) != 0:
            raise ValueError("oracle_bn254_evaluate: bad input")
        return np.split(out, np.cumsum(sizes)[:-1])

    def bench(self, circuit, witness, n_threads, proofs_per_thread, grinding_bits=10):
        w = np.ascontiguousarray(witness, dtype=np.uint64)
        arr, keep = _layers(circuit)
        t = self.lib.oracle_bn254_bench(arr, len(circuit.layers), w.shape[1], w.ctypes.data, grinding_bits,
                                        n_threads, proofs_per_thread)
        if t < 0:
            raise RuntimeError("oracle_bn254_bench failed")
        return t


class Reference:
    """The compiled, unmodified reference prover/verifier (x86-64 build only)."""

    def __init__(self, path=None):
        path = path or _build.REF_SO
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.ref_prove.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64),
                                ctypes.c_void_p]
        L.ref_verify.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
        L.ref_evaluate.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                   ctypes.c_void_p]
        L.ref_sha256.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
        sup = (ctypes.c_int * 10).in_dll(L, "ref_supported_lanes")
        self.supported_lanes = []
        for v in sup:
            if v == 0:
                break
            self.supported_lanes.append(v)

    @staticmethod
    def available():
        return os.path.exists(_build.REF_SO)

    def _loaded_layers(self, n):
        L = self.lib
        L.ref_loaded_layer.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 6
        out = []
        for k in range(n):
            nb_in, nb_out = ctypes.c_uint32(), ctypes.c_uint32()
            nm, na = ctypes.c_uint64(), ctypes.c_uint64()
            L.ref_loaded_layer(k, ctypes.byref(nb_in), ctypes.byref(nb_out), ctypes.byref(nm), ctypes.byref(na),
                               None, None)
            mul = np.empty((nm.value, 4), np.uint32)
            add = np.empty((na.value, 3), np.uint32)
            L.ref_loaded_layer(k, ctypes.byref(nb_in), ctypes.byref(nb_out), ctypes.byref(nm), ctypes.byref(na),
                               mul.ctypes.data, add.ctypes.data)
            out.append((nb_in.value, nb_out.value, mul, add))
        return out

    def circuit2_layers(self, data: bytes):
        """[(nb_input_vars, nb_output_vars, mul, add)] of the reference's CircuitRaw reader +
        Circuit::from_circuit_raw on a well-formed CIRCUIT2 file."""
        self.lib.ref_circuit2_load.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        b = np.frombuffer(bytes(data), np.uint8)
        return self._loaded_layers(self.lib.ref_circuit2_load(b.ctypes.data, b.size))

    def extracted_layers(self, mul_path: str, add_path: str):
        """The same through Circuit::load_extracted_gates on two text files."""
        self.lib.ref_extracted_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        return self._loaded_layers(self.lib.ref_extracted_load(mul_path.encode(), add_path.encode()))

    def prove(self, circuit, witness, grinding_bits=10, native=False):
        w = np.ascontiguousarray(witness, dtype=np.uint32)
        N = w.shape[1]
        R = num_repetitions(grinding_bits)
        cap = proof_size(circuit, N, R)
        proof = np.empty(cap, np.uint8)
        cv = np.empty((R, N), np.uint32)
        plen = ctypes.c_uint64()
        arr, keep = _layers(circuit)
        rc = self.lib.ref_prove(N, int(native), arr, len(circuit.layers), w.ctypes.data, grinding_bits,
                                proof.ctypes.data, cap, ctypes.byref(plen), cv.ctypes.data)
        if rc != 0:
            raise ValueError(f"ref_prove failed rc={rc} (lanes {N} supported: {self.supported_lanes})")
        return cv, proof[:plen.value].tobytes()

    def verify(self, circuit, witness, claimed_v, proof, grinding_bits=10, native=False):
        w = np.ascontiguousarray(witness, dtype=np.uint32)
        cv = np.ascontiguousarray(claimed_v, dtype=np.uint32)
        pb = np.frombuffer(bytes(proof), np.uint8)
        arr, keep = _layers(circuit)
        rc = self.lib.ref_verify(w.shape[1], int(native), arr, len(circuit.layers), w.ctypes.data, grinding_bits,
                                 pb.ctypes.data, len(pb), cv.ctypes.data)
        if rc < 0:
            raise ValueError("ref_verify: unsupported lanes")
        return rc == 1

    def evaluate(self, circuit, witness, native=False):
        w = np.ascontiguousarray(witness, dtype=np.uint32)
        N = w.shape[1]
        sizes = [1 << l.nb_input_vars for l in circuit.layers] + [1 << circuit.layers[-1].nb_output_vars]
        out = np.empty((sum(sizes), N), np.uint32)
        arr, keep = _layers(circuit)
        if self.lib.ref_evaluate(N, int(native), arr, len(circuit.layers), w.ctypes.data, out.ctypes.data) != 0:
            raise ValueError("ref_evaluate: unsupported lanes")
        return np.split(out, np.cumsum(sizes)[:-1])

    def sha256(self, data: bytes) -> bytes:
        b = np.frombuffer(bytes(data), np.uint8)
        out = np.empty(32, np.uint8)
        self.lib.ref_sha256(b.ctypes.data if len(b) else None, len(b), out.ctypes.data)
        return out.tobytes()


def _bytes_of(arr):
    a = np.ascontiguousarray(arr)
    return a, a.ctypes.data


class ReferenceBn254:
    """The reference prover/verifier templates instantiated with the BN254 type of
    oracle/bn254.h (x86-64 build only).  Witness: (rows, N, 4) uint64 limbs."""

    def __init__(self, path=None):
        path = path or _build.REF_SO
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        L = self.lib
        P, I, U64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64
        L.ref_prove_bn254.argtypes = [I, P, I, P, I, P, U64, ctypes.POINTER(U64), P]
        L.ref_verify_bn254.argtypes = [I, P, I, P, I, P, U64, P]
        L.ref_evaluate_bn254.argtypes = [I, P, I, P, P]
        L.ref_num_repetitions_bn254.argtypes = [I]
        for f in ("ref_bn254_mul", "ref_bn254_add", "ref_bn254_sub"):
            getattr(L, f).argtypes = [P, P, P]
        L.ref_bn254_reduce.argtypes = [P, P]
        sup = (ctypes.c_int * 5).in_dll(L, "ref_supported_lanes_bn254")
        self.supported_lanes = [v for v in sup if v]

    @staticmethod
    def proof_size(circuit, n_copies):
        rows = sum(6 * l.nb_input_vars + 2 for l in circuit.layers)
        return (1 << circuit.layers[0].nb_input_vars) * n_copies * 32 + 32 + rows * n_copies * 32

    def prove(self, circuit, witness, grinding_bits=10):
        w, wp = _bytes_of(np.asarray(witness, dtype=np.uint64))
        N = w.shape[1]
        cap = self.proof_size(circuit, N)
        proof = np.empty(cap, np.uint8)
        cv = np.empty((1, N, 4), np.uint64)
        plen = ctypes.c_uint64()
        arr, keep = _layers(circuit)
        rc = self.lib.ref_prove_bn254(N, arr, len(circuit.layers), wp, grinding_bits, proof.ctypes.data, cap,
                                      ctypes.byref(plen), cv.ctypes.data)
        if rc != 0:
            raise ValueError(f"ref_prove_bn254 failed rc={rc}")
        return cv, proof[:plen.value].tobytes()

    def verify(self, circuit, witness, claimed_v, proof, grinding_bits=10):
        w, wp = _bytes_of(np.asarray(witness, dtype=np.uint64))
        cv, cvp = _bytes_of(np.asarray(claimed_v, dtype=np.uint64))
        pb = np.frombuffer(bytes(proof), np.uint8)
        arr, keep = _layers(circuit)
        rc = self.lib.ref_verify_bn254(w.shape[1], arr, len(circuit.layers), wp, grinding_bits, pb.ctypes.data,
                                       len(pb), cvp)
        if rc < 0:
            raise ValueError("ref_verify_bn254: unsupported lanes")
        return rc == 1

    def evaluate(self, circuit, witness):
        w, wp = _bytes_of(np.asarray(witness, dtype=np.uint64))
        N = w.shape[1]
        sizes = [1 << l.nb_input_vars for l in circuit.layers] + [1 << circuit.layers[-1].nb_output_vars]
        out = np.empty((sum(sizes), N, 4), np.uint64)
        arr, keep = _layers(circuit)
        if self.lib.ref_evaluate_bn254(N, arr, len(circuit.layers), wp, out.ctypes.data) != 0:
            raise ValueError("ref_evaluate_bn254: unsupported lanes")
        return np.split(out, np.cumsum(sizes)[:-1])

    def field_op(self, name, a: int, b: int = 0) -> int:
        ab = a.to_bytes(32, "little")
        bb = b.to_bytes(32, "little")
        out = ctypes.create_string_buffer(32)
        if name == "reduce":
            self.lib.ref_bn254_reduce(ab, out)
        else:
            getattr(self.lib, "ref_bn254_" + name)(ab, bb, out)
        return int.from_bytes(out.raw, "little")
