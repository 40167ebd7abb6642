"""Python mirror of the reference prover API on top of the C ABI.

Reference (PolyhedraZK/Expander-cpp)                       here
  Config (include/configuration/config.hpp:26-86)        Config
  Prover(config).prepare_mem(circuit); prove(circuit)    Prover(config).prepare_mem(circuit); prove(circuit)
    (include/LinearGKR/LinearGKR.hpp:34-91)                -> (claimed_v (R, N) uint32, Proof)
  Circuit::evaluate (include/circuit/circuit.hpp:273-280) Context.evaluate / Prover.evaluate
  Proof (include/fiat_shamir/transcript.hpp:13-85)       Proof (bytes + write/read of the length-prefixed file)

The circuit input (the reference's layers[0].input_layer_vals) is a (2^n, N) uint32 array
set with Circuit.set_input or passed to prove() directly.
"""
import ctypes
import os

import numpy as np

from . import _lib
from .circuit import Circuit


class Config:
    """Config of the reference: 100-bit security, RAW commitment, field M31 (default) or BN254,
    transcript hash SHA256 (default, the reference's) or Keccak256 (config.hpp:12-24,40-86)."""

    def __init__(self, grinding_bits: int = 10, field_type: str = "M31", FS_hash: str = "SHA256"):
        if field_type not in ("M31", "BN254"):
            raise ValueError(f"unsupported field_type {field_type!r} (M31 or BN254)")
        if FS_hash not in _lib.FS_HASHES:
            raise ValueError(f"unsupported FS_hash {FS_hash!r} (SHA256 or Keccak256)")
        self.security_bits = 100
        self.grinding_bits = int(grinding_bits)
        self.field_type = field_type
        self.field_size = 254 if field_type == "BN254" else 31
        self.PC_type = "Raw"
        self.FS_hash = FS_hash

    def get_num_repetitions(self) -> int:
        return _lib.load().gkrgpu_num_repetitions_field(_lib.FIELDS[self.field_type], self.grinding_bits)


def _table(field: str, values):
    """A value table in the C layout: M31 (rows, N) uint32; BN254 (rows, N, 4) uint64 limbs
    (little-endian, i.e. the 32 canonical bytes of each element)."""
    if field == "BN254":
        a = np.ascontiguousarray(values, dtype=np.uint64)
        if a.ndim != 3 or a.shape[2] != 4:
            raise ValueError("a BN254 table is a (rows, N, 4) uint64 array")
        return a
    a = np.ascontiguousarray(values, dtype=np.uint32)
    if a.ndim != 2:
        raise ValueError("an M31 table is a (rows, N) uint32 array")
    return a


def _empty(field: str, rows: int, n: int):
    return np.empty((rows, n, 4), np.uint64) if field == "BN254" else np.empty((rows, n), np.uint32)


class Proof:
    """Proof bytes (the transcript).  write/read use the reference's file format: a 4-byte
    little-endian length then the bytes (transcript.hpp:54-84)."""

    def __init__(self, data: bytes = b""):
        self.bytes = bytes(data)

    def __len__(self):
        return len(self.bytes)

    def __eq__(self, other):
        return isinstance(other, Proof) and self.bytes == other.bytes

    def write(self, path):
        """Proof::write_and_compress without the tar step (gkrgpu_proof_write)."""
        b = np.frombuffer(self.bytes, np.uint8)
        _lib.check(_lib.load().gkrgpu_proof_write(os.fsencode(path), b.ctypes.data if b.size else None, b.size))

    @staticmethod
    def read(path):
        """Proof::read_proof (gkrgpu_proof_read)."""
        lib = _lib.load()
        n = ctypes.c_uint64()
        _lib.check(lib.gkrgpu_proof_read(os.fsencode(path), None, 0, ctypes.byref(n)))
        buf = np.empty(max(n.value, 1), np.uint8)
        _lib.check(lib.gkrgpu_proof_read(os.fsencode(path), buf.ctypes.data, buf.nbytes, ctypes.byref(n)))
        return Proof(buf[:n.value].tobytes())


class DeviceCircuit:
    """A circuit's wiring resident on the device (gkrgpu_circuit_load_field)."""

    def __init__(self, ctx: "Context", circuit: Circuit, field: str = "M31"):
        lib = _lib.load()
        circuit.validate(field)
        self.ctx = ctx
        self.field = field
        self.n_layers = len(circuit.layers)
        self.log_input_size = circuit.log_input_size
        self.nb_output_vars = circuit.layers[-1].nb_output_vars
        descs = (_lib.LayerDesc * self.n_layers)()
        keep = []
        for k, l in enumerate(circuit.layers):
            m = np.ascontiguousarray(l.mul, dtype=np.uint32)
            a = np.ascontiguousarray(l.add, dtype=np.uint32)
            keep += [m, a]
            descs[k] = _lib.LayerDesc(l.nb_output_vars, l.nb_input_vars, m.shape[0], a.shape[0],
                                      m.ctypes.data if m.size else None, a.ctypes.data if a.size else None)
        h = ctypes.c_void_p()
        _lib.check(lib.gkrgpu_circuit_load_field(ctx.handle, descs, self.n_layers, _lib.FIELDS[field], ctypes.byref(h)))
        self.handle = h

    def proof_size(self, n_copies, grinding_bits=10):
        return _lib.load().gkrgpu_proof_size(self.handle, n_copies, grinding_bits)

    def num_repetitions(self, grinding_bits=10):
        return _lib.load().gkrgpu_num_repetitions_field(_lib.FIELDS[self.field], grinding_bits)

    def free(self):
        if getattr(self, "handle", None):
            _lib.load().gkrgpu_circuit_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """One CUDA device, its stream and the reusable prover workspace (gkrgpu_create)."""

    def __init__(self, device: int = 0):
        lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(lib.gkrgpu_create(device, ctypes.byref(h)))
        self.handle = h
        self.device = device
        self.fs_hash = "SHA256"

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().gkrgpu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, circuit: Circuit, field: str = "M31") -> DeviceCircuit:
        return DeviceCircuit(self, circuit, field)

    def set_fs_hash(self, name: str):
        """Transcript hash of later proofs and verifications: "SHA256" (the reference's) or
        "Keccak256" (gkrgpu_set_fs_hash; waits for queued proofs)."""
        if name not in _lib.FS_HASHES:
            raise ValueError(f"unsupported FS_hash {name!r} (SHA256 or Keccak256)")
        if name != self.fs_hash:
            _lib.check(_lib.load().gkrgpu_set_fs_hash(self.handle, _lib.FS_HASHES[name]))
            self.fs_hash = name

    def evaluate(self, dc: DeviceCircuit, witness, all_layers=False):
        """Circuit::evaluate on the device; returns the output rows, or with all_layers every
        layer's input rows followed by the output rows, as one (rows, N) table."""
        lib = _lib.load()
        w = _table(dc.field, witness)
        rows = lib.gkrgpu_value_rows(dc.handle, int(all_layers))
        out = _empty(dc.field, rows, w.shape[1])
        _lib.check(lib.gkrgpu_evaluate(self.handle, dc.handle, w.shape[1], w.ctypes.data, out.ctypes.data,
                                       int(all_layers)))
        return out

    def prove(self, dc: DeviceCircuit, witness, grinding_bits=10, out=None):
        """Prover::prove; returns (claimed_v (R, N) table, proof bytes).  `out` may be a
        preallocated uint8 buffer of at least proof_size bytes (e.g. pinned host memory)."""
        lib = _lib.load()
        w = _table(dc.field, witness)
        N = w.shape[1]
        cap = dc.proof_size(N, grinding_bits)
        buf = np.empty(cap, np.uint8) if out is None else out
        cv = _empty(dc.field, dc.num_repetitions(grinding_bits), N)
        plen = ctypes.c_uint64()
        _lib.check(lib.gkrgpu_prove(self.handle, dc.handle, N, grinding_bits, w.ctypes.data, buf.ctypes.data,
                                    buf.nbytes, ctypes.byref(plen), cv.ctypes.data))
        return cv, (buf[:plen.value].tobytes() if out is None else plen.value)

    def prove_device(self, dc: DeviceCircuit, d_input: int, n_copies: int, out_buf, grinding_bits=10):
        """Prover::prove with the input already in device memory at address d_input."""
        lib = _lib.load()
        cv = _empty(dc.field, dc.num_repetitions(grinding_bits), n_copies)
        plen = ctypes.c_uint64()
        _lib.check(lib.gkrgpu_prove_device(self.handle, dc.handle, n_copies, grinding_bits, ctypes.c_void_p(d_input),
                                           out_buf.ctypes.data, out_buf.nbytes, ctypes.byref(plen), cv.ctypes.data))
        return cv, plen.value

    def submit(self, dc: DeviceCircuit, witness, proof_buf, claimed_buf, grinding_bits=10, d_input=None,
               marker=-1):
        """gkrgpu_prove_submit: queues one proof and returns a Job.  The witness (host array)
        or d_input (device address), proof_buf and claimed_buf must outlive the job."""
        lib = _lib.load()
        h = ctypes.c_void_p()
        if d_input is not None:
            src, on_dev, n, keep = ctypes.c_void_p(d_input), 1, claimed_buf.shape[1], None
        else:
            keep = _table(dc.field, witness)
            src, on_dev, n = keep.ctypes.data, 0, keep.shape[1]
        _lib.check(lib.gkrgpu_prove_submit(self.handle, dc.handle, n, grinding_bits, src, on_dev,
                                           proof_buf.ctypes.data, proof_buf.nbytes, claimed_buf.ctypes.data, marker,
                                           ctypes.byref(h)))
        return Job(h, (keep, proof_buf, claimed_buf))

    def submit_resident(self, dc: DeviceCircuit, witness, d_input: int, proof_buf, claimed_buf, grinding_bits=10,
                        marker=-1):
        """gkrgpu_prove_submit_resident: the witness both in host memory (hashed for the RAW
        commitment) and resident on the device at d_input (computed from); no input copy."""
        lib = _lib.load()
        h = ctypes.c_void_p()
        keep = _table(dc.field, witness)
        _lib.check(lib.gkrgpu_prove_submit_resident(self.handle, dc.handle, claimed_buf.shape[1], grinding_bits,
                                                    keep.ctypes.data, ctypes.c_void_p(d_input),
                                                    proof_buf.ctypes.data, proof_buf.nbytes, claimed_buf.ctypes.data,
                                                    marker, ctypes.byref(h)))
        return Job(h, (keep, proof_buf, claimed_buf))

    def upload(self, d_dst: int, host_array):
        """gkrgpu_upload: host -> device copy that does not wait for queued proofs."""
        a = np.ascontiguousarray(host_array)
        _lib.check(_lib.load().gkrgpu_upload(self.handle, ctypes.c_void_p(d_dst), a.ctypes.data, a.nbytes))

    def set_round_tail(self, enabled: bool):
        """Phase tails in one persistent launch (default) or one launch per round."""
        _lib.check(_lib.load().gkrgpu_set_round_tail(self.handle, int(enabled)))

    def check_device_wait(self, timeout_us: int):
        """gkrgpu_check_device_wait: (expired, rounds_published) of a tail whose second
        challenge never comes."""
        e, r = ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.load().gkrgpu_check_device_wait(self.handle, timeout_us, ctypes.byref(e), ctypes.byref(r)))
        return bool(e.value), r.value

    def set_host_threads(self, threads=0):
        """Host threads for host stages (commitment hashing); 0 restores the default."""
        _lib.check(_lib.load().gkrgpu_set_host_threads(self.handle, threads))

    def wait(self, job: "Job") -> int:
        """gkrgpu_prove_wait: blocks until the job is done; returns the proof length."""
        plen = ctypes.c_uint64()
        h, job.handle = job.handle, None
        _lib.check(_lib.load().gkrgpu_prove_wait(h, ctypes.byref(plen)))
        return plen.value

    def verify(self, dc: DeviceCircuit, proof, claimed_v, grinding_bits=10) -> bool:
        """Verifier::verify of an M31 proof (gkrgpu_verify): True when the reference verifier
        accepts.  claimed_v is the (R, N) uint32 table the prover returned."""
        cv = _table(dc.field, claimed_v)
        pb = np.frombuffer(bytes(proof), np.uint8)
        ok = ctypes.c_int()
        _lib.check(_lib.load().gkrgpu_verify(self.handle, dc.handle, cv.shape[1], grinding_bits,
                                             pb.ctypes.data if pb.size else None, pb.size, cv.ctypes.data,
                                             ctypes.byref(ok)))
        return ok.value == 1

    def eval_multilinear(self, d_evals: int, nb_vars: int, n_copies: int, points):
        """eval_multilinear of the device table at d_evals (2^nb_vars rows) at 1..3 points;
        returns (n_points, n_copies) uint32."""
        pts = np.ascontiguousarray(np.atleast_2d(points), dtype=np.uint32)
        out = np.empty((pts.shape[0], n_copies), np.uint32)
        _lib.check(_lib.load().gkrgpu_eval_multilinear(self.handle, ctypes.c_void_p(d_evals), nb_vars, n_copies,
                                                       pts.ctypes.data, pts.shape[0], out.ctypes.data))
        return out

    def set_timing(self, enabled: bool):
        _lib.check(_lib.load().gkrgpu_set_timing(self.handle, int(enabled)))

    def reset_stats(self):
        _lib.check(_lib.load().gkrgpu_reset_stats(self.handle))

    def kernel_stats(self):
        lib = _lib.load()
        arr = (_lib.KernelStat * 32)()
        n = lib.gkrgpu_kernel_stats(self.handle, arr, 32)
        return {arr[i].name.decode(): {"launches": arr[i].launches, "ms": arr[i].total_ms,
                                       "bytes": arr[i].algorithmic_bytes} for i in range(min(n, 32))}

    def set_tile(self, threads_per_row=0, block=0, ctas=0):
        _lib.check(_lib.load().gkrgpu_set_tile(self.handle, threads_per_row, block, ctas))

    def autotune(self, dc: DeviceCircuit, witness=None, n_copies=None, d_input=None, grinding_bits=10):
        """gkrgpu_autotune: picks each kernel kind's row tile by timing whole proofs.  Returns
        {kernel: {"threads_per_row", "ctas", "ms"}}."""
        lib = _lib.load()
        arr = (_lib.TileChoice * 32)()
        if d_input is not None:
            src, on_dev, n, keep = ctypes.c_void_p(d_input), 1, n_copies, None
        else:
            keep = _table(dc.field, witness)
            src, on_dev, n = keep.ctypes.data, 0, keep.shape[1]
        _lib.check(lib.gkrgpu_autotune(self.handle, dc.handle, n, grinding_bits, src, on_dev, arr, 32))
        names = list(self.kernel_stats().keys())
        return {names[i]: {"threads_per_row": arr[i].threads_per_row, "ctas": arr[i].ctas, "ms": arr[i].ms}
                for i in range(len(names))}

    def set_concurrency(self, lanes=0, hbm_budget_bytes=0):
        """Device stages of up to `lanes` proofs run at once under an HBM budget."""
        _lib.check(_lib.load().gkrgpu_set_concurrency(self.handle, lanes, hbm_budget_bytes))

    def memory_stats(self):
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(_lib.load().gkrgpu_memory_stats(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"in_use": a.value, "peak": b.value, "budget": c.value}

    def mark(self, slot: int):
        """Records timing marker `slot` on the context's stream."""
        _lib.check(_lib.load().gkrgpu_mark(self.handle, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = ctypes.c_double()
        _lib.check(_lib.load().gkrgpu_elapsed_ms(self.handle, a, b, ctypes.byref(ms)))
        return ms.value

    def transfer_stats(self):
        h, d = ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(_lib.load().gkrgpu_transfer_stats(self.handle, ctypes.byref(h), ctypes.byref(d)))
        return h.value, d.value


class Job:
    """A queued proof (gkrgpu_job); keeps its buffers alive until waited on.  A job dropped
    without Context.wait is waited for here, so its buffers are never freed while the library
    still copies into them."""

    def __init__(self, handle, buffers):
        self.handle = handle
        self.buffers = buffers

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h:
            try:
                _lib.load().gkrgpu_prove_wait(h, ctypes.byref(ctypes.c_uint64()))
            except Exception:
                pass


class HostBuffer:
    """Pinned host memory (gkrgpu_host_alloc) viewed as a numpy array."""

    def __init__(self, nbytes: int, dtype=np.uint8):
        p = ctypes.c_void_p()
        _lib.check(_lib.load().gkrgpu_host_alloc(nbytes, ctypes.byref(p)))
        self.ptr = p.value
        self.nbytes = nbytes
        raw = (ctypes.c_uint8 * nbytes).from_address(self.ptr)
        raw._owner = self  # views of .array keep the pinned block alive
        self.array = np.ctypeslib.as_array(raw).view(dtype)

    def free(self):
        if self.ptr:
            self.array = None
            _lib.load().gkrgpu_host_free(ctypes.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class DeviceBuffer:
    """Device memory owned through a context (gkrgpu_device_alloc)."""

    def __init__(self, ctx: Context, nbytes: int):
        p = ctypes.c_void_p()
        _lib.check(_lib.load().gkrgpu_device_alloc(ctx.handle, nbytes, ctypes.byref(p)))
        self.ctx, self.ptr, self.nbytes = ctx, p.value, nbytes

    def upload(self, host_array):
        a = np.ascontiguousarray(host_array)
        _lib.check(_lib.load().gkrgpu_memcpy_h2d(self.ctx.handle, ctypes.c_void_p(self.ptr), a.ctypes.data, a.nbytes))

    def free(self):
        if self.ptr:
            _lib.load().gkrgpu_device_free(self.ctx.handle, ctypes.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Prover:
    """gkr::Prover (include/LinearGKR/LinearGKR.hpp:34-91) on the GPU."""

    def __init__(self, config: Config = None, ctx: Context = None):
        self.config = config or Config()
        self.ctx = ctx or Context(0)
        self._dc = None
        self._circuit = None

    def prepare_mem(self, circuit: Circuit):
        """Uploads the circuit's wiring (the reference allocates its scratch pads here)."""
        if self._circuit is not circuit:
            self._dc = self.ctx.load(circuit, self.config.field_type)
            self._circuit = circuit

    def prove(self, circuit: Circuit, witness=None):
        if self._circuit is not circuit:
            self.prepare_mem(circuit)
        w = circuit.input_values if witness is None else witness
        if w is None:
            raise ValueError("no circuit input: call circuit.set_input(values) or pass witness")
        self.ctx.set_fs_hash(self.config.FS_hash)
        cv, proof = self.ctx.prove(self._dc, w, self.config.grinding_bits)
        return cv, Proof(proof)


class Verifier:
    """gkr::Verifier (include/LinearGKR/LinearGKR.hpp:92-149) with its device-side parts on the
    GPU (gkrgpu_verify); M31 and BN254 circuits."""

    def __init__(self, config: Config = None, ctx: Context = None):
        self.config = config or Config()
        self.ctx = ctx or Context(0)
        self._dc = None
        self._circuit = None

    def verify(self, circuit: Circuit, claimed_v, proof) -> bool:
        if self._circuit is not circuit:
            self._dc = self.ctx.load(circuit, self.config.field_type)
            self._circuit = circuit
        data = proof.bytes if isinstance(proof, Proof) else proof
        self.ctx.set_fs_hash(self.config.FS_hash)
        return self.ctx.verify(self._dc, data, claimed_v, self.config.grinding_bits)
