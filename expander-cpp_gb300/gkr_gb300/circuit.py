"""Layered-circuit model and seeded synthetic circuit generators.

Mirrors the reference's circuit types (include/circuit/circuit.hpp):

* ``Gate<F,2>`` (o_id, i_ids[2], coef)  -> one row of ``CircuitLayer.mul`` (uint32 x 4)
* ``Gate<F,1>`` (o_id, i_ids[1], coef)  -> one row of ``CircuitLayer.add`` (uint32 x 3)
* ``CircuitLayer`` (nb_output_vars, nb_input_vars, mul, add)  circuit.hpp:68-116
* ``Circuit`` (layers, layer 0 is the input side)              circuit.hpp:118-305

Field elements are M31 (p = 2^31 - 1) stored canonical in [0, p).  A witness for N
data-parallel copies is a (2^nb_input_vars(layer 0), N) uint32 array: row i holds the
N lanes of input i, the byte layout of VectorizedM31::to_bytes (M31.hpp:420-426).
"""
from __future__ import annotations

import numpy as np

P = 2147483647  # M31 modulus, include/field/M31.hpp:20


class CircuitLayer:
    """One layer: out[o] = sum_mul v[i0]*v[i1]*c + sum_add v[i0]*c (circuit.hpp:92-105)."""

    def __init__(self, nb_output_vars: int, nb_input_vars: int, mul=None, add=None):
        self.nb_output_vars = int(nb_output_vars)
        self.nb_input_vars = int(nb_input_vars)
        self.mul = np.ascontiguousarray(np.zeros((0, 4), np.uint32) if mul is None else mul, dtype=np.uint32)
        self.add = np.ascontiguousarray(np.zeros((0, 3), np.uint32) if add is None else add, dtype=np.uint32)
        if self.mul.ndim != 2 or self.mul.shape[1] != 4:
            raise ValueError("mul gates must be an (n, 4) array of (o_id, i0, i1, coef)")
        if self.add.ndim != 2 or self.add.shape[1] != 3:
            raise ValueError("add gates must be an (n, 3) array of (o_id, i0, coef)")

    @property
    def nb_mul_gates(self) -> int:
        return int(self.mul.shape[0])

    @property
    def nb_add_gates(self) -> int:
        return int(self.add.shape[0])

    @staticmethod
    def random(nb_output_vars: int, nb_input_vars: int) -> "CircuitLayer":
        """Deterministic wiring of CircuitLayer::random / SparseCircuitConnection::random
        (circuit.hpp:40-65,80-90): output i <- inputs i mod I and (i + O) mod I, coef 1,
        one mul and one add gate per output."""
        O, I = 1 << nb_output_vars, 1 << nb_input_vars
        o = np.arange(O, dtype=np.uint64)
        mul = np.stack([o, o % I, (o + O) % I, np.ones(O, np.uint64)], axis=1).astype(np.uint32)
        add = np.stack([o, o % I, np.ones(O, np.uint64)], axis=1).astype(np.uint32)
        return CircuitLayer(nb_output_vars, nb_input_vars, mul, add)


class Circuit:
    """An ordered list of layers; layers[0] reads the circuit input (circuit.hpp:118-122)."""

    def __init__(self, layers=None):
        self.layers: list[CircuitLayer] = list(layers or [])
        self.input_values = None  # layers[0].input_layer_vals of the reference

    @staticmethod
    def from_circuit2(data) -> "Circuit":
        """A CIRCUIT2 file (path or bytes) as CircuitRaw + Circuit::from_circuit_raw load it
        (include/circuit/circuit_raw.hpp:511-568, include/circuit/circuit.hpp:217-251),
        parsed by the native library (gkrgpu_circuit2_parse)."""
        if not isinstance(data, (bytes, bytearray, memoryview)):
            with open(data, "rb") as f:
                data = f.read()
        b = np.frombuffer(bytes(data), np.uint8)
        return Circuit._from_parsed(lambda lib, h: lib.gkrgpu_circuit2_parse(b.ctypes.data if b.size else None,
                                                                            b.size, h))

    @staticmethod
    def from_extracted(mul, add) -> "Circuit":
        """The text gate lists of Circuit::load_extracted_gates (circuit.hpp:152-215): paths
        or the file contents as str/bytes (gkrgpu_extracted_parse)."""
        def text(x):
            if isinstance(x, (bytes, bytearray)):
                return bytes(x)
            if isinstance(x, str) and ("\n" in x or not x.strip()):
                return x.encode()
            with open(x, "rb") as f:
                return f.read()
        m, a = text(mul), text(add)
        return Circuit._from_parsed(lambda lib, h: lib.gkrgpu_extracted_parse(m, len(m), a, len(a), h))

    @staticmethod
    def _from_parsed(parse) -> "Circuit":
        import ctypes

        from . import _lib
        lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(parse(lib, ctypes.byref(h)))
        try:
            layers = []
            for k in range(lib.gkrgpu_parsed_layers(h)):
                d = _lib.LayerDesc()
                _lib.check(lib.gkrgpu_parsed_layer(h, k, ctypes.byref(d)))
                mul = np.ctypeslib.as_array(ctypes.cast(d.mul, ctypes.POINTER(ctypes.c_uint32)), (d.n_mul, 4)).copy() \
                    if d.n_mul else None
                add = np.ctypeslib.as_array(ctypes.cast(d.add, ctypes.POINTER(ctypes.c_uint32)), (d.n_add, 3)).copy() \
                    if d.n_add else None
                layers.append(CircuitLayer(d.nb_output_vars, d.nb_input_vars, mul, add))
            return Circuit(layers)
        finally:
            lib.gkrgpu_parsed_free(h)

    def set_input(self, values) -> None:
        """Sets the circuit input: a (2^nb_input_vars(layer 0), N) array of canonical M31."""
        v = np.ascontiguousarray(values, dtype=np.uint32)
        if v.ndim != 2 or v.shape[0] != (1 << self.log_input_size):
            raise ValueError(f"input must have shape (2^{self.log_input_size}, N)")
        self.input_values = v

    @property
    def log_input_size(self) -> int:
        return self.layers[0].nb_input_vars

    @property
    def nb_mul_gates(self) -> int:
        return sum(l.nb_mul_gates for l in self.layers)

    @property
    def nb_add_gates(self) -> int:
        return sum(l.nb_add_gates for l in self.layers)

    def validate(self, field: str = "M31") -> None:
        """Raises ValueError for inconsistent widths, out-of-range ids or coefficients (M31
        coefficients must be below p; every uint32 is a canonical BN254 coefficient)."""
        limit = 1 << 32 if field == "BN254" else P
        if not self.layers:
            raise ValueError("circuit has no layers")
        for k, l in enumerate(self.layers):
            if not (1 <= l.nb_input_vars <= 30 and 0 <= l.nb_output_vars <= 30):
                raise ValueError(f"layer {k}: nb_input_vars must be in [1, 30], nb_output_vars in [0, 30]")
            if k + 1 < len(self.layers) and l.nb_output_vars != self.layers[k + 1].nb_input_vars:
                raise ValueError(f"layer {k}: nb_output_vars != nb_input_vars of layer {k + 1}")
            O, I = 1 << l.nb_output_vars, 1 << l.nb_input_vars
            if l.nb_mul_gates and (l.mul[:, 0].max() >= O or l.mul[:, 1:3].max() >= I or l.mul[:, 3].max() >= limit):
                raise ValueError(f"layer {k}: mul gate id or coefficient out of range")
            if l.nb_add_gates and (l.add[:, 0].max() >= O or l.add[:, 1].max() >= I or l.add[:, 2].max() >= limit):
                raise ValueError(f"layer {k}: add gate id or coefficient out of range")

    def proof_size(self, n_copies: int, reps: int = 3) -> int:
        """Bytes of Prover::prove's proof: RAW commitment + 32 grinding bytes + per layer
        R*(6n + 2) vectors of 4N bytes (include/LinearGKR/sumcheck.hpp:72-103)."""
        rows = sum(reps * (6 * l.nb_input_vars + 2) for l in self.layers)
        return (1 << self.log_input_size) * n_copies * 4 + 32 + rows * n_copies * 4


class Stream:
    """Counter-based SplitMix64 stream: the same seed gives the same values on every
    platform and numpy version (the synthetic workloads and golden fixtures rely on it)."""

    GAMMA = np.uint64(0x9E3779B97F4A7C15)

    def __init__(self, seed: int):
        self.key = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self.ctr = 0

    def u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            i = np.arange(self.ctr + 1, self.ctr + 1 + n, dtype=np.uint64)
            self.ctr += n
            z = self.key + i * self.GAMMA
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            return z ^ (z >> np.uint64(31))

    def below(self, n: int, bound) -> np.ndarray:
        """n integers in [0, bound) (bound may be an array), by 32x32-bit multiply-shift."""
        hi = self.u64(n) >> np.uint64(32)
        return (hi * np.asarray(bound, dtype=np.uint64)) >> np.uint64(32)

    def uniform(self, n: int) -> np.ndarray:
        return (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))

    def field(self, n: int) -> np.ndarray:
        """n canonical M31 elements in [0, p)."""
        return self.below(n, P).astype(np.uint32)


def _coefs(st, n, p_one=0.5):
    c = st.below(n, P)
    c[st.uniform(n) < p_one] = 1
    return c


def _wire(st, o, O, I, n, p_local, window):
    """Input ids for outputs o: local to the aligned window containing floor(o*I/O) with
    probability p_local, uniform over [0, I) otherwise."""
    u = st.below(n, I)
    if p_local <= 0.0:
        return u
    w = min(window, I)
    centre = (o.astype(np.uint64) * np.uint64(I)) // np.uint64(O)
    base = (centre // np.uint64(w)) * np.uint64(w)
    loc = base + st.below(n, w)
    pick = st.uniform(n) < p_local
    return np.where(pick, loc, u)


def random_layer(st, nb_output_vars, nb_input_vars, p_mul=0.5, p_local=0.0, window=1 << 12, p_coef_one=0.5):
    """One random layer: each output is a fan-in-2 mul gate with probability p_mul, else a
    fan-in-2 add gate (two Gate<F,1> entries with the same o_id, docs/doc.md)."""
    O, I = 1 << nb_output_vars, 1 << nb_input_vars
    is_mul = st.uniform(O) < p_mul
    mo = np.nonzero(is_mul)[0].astype(np.uint64)
    ao = np.nonzero(~is_mul)[0].astype(np.uint64)
    nm, na = len(mo), len(ao)
    mul = np.stack([mo, _wire(st, mo, O, I, nm, p_local, window), _wire(st, mo, O, I, nm, p_local, window),
                    _coefs(st, nm, p_coef_one)], axis=1).astype(np.uint32)
    ao2 = np.repeat(ao, 2)
    add = np.stack([ao2, _wire(st, ao2, O, I, 2 * na, p_local, window), _coefs(st, 2 * na, p_coef_one)],
                   axis=1).astype(np.uint32)
    return CircuitLayer(nb_output_vars, nb_input_vars, mul.reshape(-1, 4), add.reshape(-1, 3))


def random_circuit(seed, widths, p_mul=0.5, p_local=0.0, window=1 << 12):
    """Layered circuit with layer l mapping 2^widths[l] inputs to 2^widths[l+1] outputs."""
    st = Stream(seed)
    return Circuit([random_layer(st, widths[l + 1], widths[l], p_mul, p_local, window) for l in range(len(widths) - 1)])


def random_witness(seed, nb_input_vars, n_copies, out=None):
    """Uniform M31 witness, shape (2^nb_input_vars, n_copies), canonical.  Generated in
    chunks (so a 1 GiB witness does not need several GiB of temporaries); `out` may be a
    preallocated uint32 array of that shape (e.g. pinned host memory)."""
    rows = 1 << nb_input_vars
    n = rows * n_copies
    res = np.empty((rows, n_copies), np.uint32) if out is None else out
    flat = res.reshape(-1)
    st = Stream(seed ^ 0x5EED5EED5EED5EED)
    chunk = 1 << 22
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        flat[s:s + m] = st.field(m)
    return res


BN254_R = 0x30644E72E131A029B85045B68181585D2833E84879B9709143E1F593F0000001  # BN254 scalar field modulus
_BN254_TOP = np.uint64(0x30644E72E131A029)


def random_witness_bn254(seed, nb_input_vars, n_copies):
    """BN254 witness of canonical elements, shape (2^nb_input_vars, n_copies, 4) uint64:
    the 4 little-endian 64-bit limbs of each element (its 32-byte encoding).  The top limb
    is drawn below r's top limb, so every value is < r."""
    rows = 1 << nb_input_vars
    st = Stream(seed ^ 0xB254B254B254B254)
    limbs = st.u64(rows * n_copies * 4).reshape(rows, n_copies, 4)
    limbs[..., 3] %= _BN254_TOP
    return limbs


def bn254_values(arr) -> list:
    """Python integers of a (..., 4) uint64 limb array (flattened)."""
    a = np.asarray(arr, dtype=np.uint64).reshape(-1, 4)
    return [int(x[0]) | (int(x[1]) << 64) | (int(x[2]) << 128) | (int(x[3]) << 192) for x in a]


def uniform_circuit(seed, depth, width, p_mul=0.5):
    """`depth` layers of 2^width gates with uniform wiring, generated in one vectorised pass
    (the mixed-batch workload builds hundreds of these)."""
    st = Stream(seed)
    O = I = 1 << width
    is_mul = st.uniform(depth * O).reshape(depth, O) < p_mul
    layers = []
    for l in range(depth):
        mo = np.nonzero(is_mul[l])[0].astype(np.uint64)
        ao = np.repeat(np.nonzero(~is_mul[l])[0].astype(np.uint64), 2)
        nm, na = len(mo), len(ao)
        r = st.below(2 * nm + na, I)
        c = _coefs(st, nm + na)
        mul = np.stack([mo, r[:nm], r[nm:2 * nm], c[:nm]], axis=1).astype(np.uint32)
        add = np.stack([ao, r[2 * nm:], c[nm:]], axis=1).astype(np.uint32)
        layers.append(CircuitLayer(width, width, mul, add))
    return Circuit(layers)


def mixed_batch_specs(seed=3, n_proofs=512, depth=(4, 24), width=(8, 18), copies=(16, 256)):
    """Per-proof (seed, depth, width, copies) of the mixed batched workload: depth and width
    exponent uniform in their ranges, copies uniform in the range rounded down to a multiple
    of 16."""
    st = Stream(seed)
    d = depth[0] + st.below(n_proofs, depth[1] - depth[0] + 1)
    k = width[0] + st.below(n_proofs, width[1] - width[0] + 1)
    n = copies[0] + st.below(n_proofs, copies[1] - copies[0] + 1)
    n = np.maximum(16, (n // 16) * 16)
    return [(int(seed * 100003 + i), int(d[i]), int(k[i]), int(n[i])) for i in range(n_proofs)]


# ---------------------------------------------------------------- named workloads

def config1_circuit(seed=1234, n_layers=8, width=10):
    """Small plain workload: 8 layers of 2^10 gates, 50% mul, uniform wiring."""
    return random_circuit(seed, [width] * (n_layers + 1), p_mul=0.5)


def config2_circuit(seed=2024, n_layers=24, wide=20, narrow=18):
    """Large Keccak-like workload: 24 layers whose widths alternate 2^18 / 2^20 (the input
    layer is 2^18 so the RAW commitment stays below 4 GiB at 1024 copies), 60% mul, wiring
    local to 2^12-gate windows with probability 0.8."""
    widths = [narrow if l % 2 == 0 else wide for l in range(n_layers + 1)]
    return random_circuit(seed, widths, p_mul=0.6, p_local=0.8, window=1 << 12)


def config4_circuit(seed=4254, n_layers=16, width=16):
    """BN254 plain workload: 16 layers of 2^16 gates, 50% mul / 50% add, uniform wiring."""
    return uniform_circuit(seed, n_layers, width, p_mul=0.5)
