"""Writers of the reference's circuit file formats for the loader tests: the binary CIRCUIT2
segment format (the layout CircuitRaw::operator>> reads, include/circuit/circuit_raw.hpp:
275-352, 511-568, with 32-byte field elements as the compiler writes them) and the text gate
lists of Circuit::load_extracted_gates (include/circuit/circuit.hpp:152-215)."""
import struct

import numpy as np

from gkr_gb300 import circuit as gc

MAGIC = 3626604230490605891


def _fe(x):
    return struct.pack("<I", x & 0xFFFFFFFF) + bytes(28)


def segment_bytes(seg):
    """seg: dict(i_len, o_len, children=[(sid, [(i_off, o_off), ...])], mul=[(in0, in1, out, c)],
    add=[(in0, out, c)], const=[(out, c)], rand=[gate index, ...])."""
    b = struct.pack("<QQ", seg["i_len"], seg["o_len"])
    ch = seg.get("children", [])
    b += struct.pack("<Q", len(ch))
    for sid, allocs in ch:
        b += struct.pack("<QQ", sid, len(allocs))
        for io, oo in allocs:
            b += struct.pack("<QQ", io, oo)
    mul = seg.get("mul", [])
    b += struct.pack("<Q", len(mul))
    for in0, in1, out, c in mul:
        b += struct.pack("<QQQ", in0, in1, out) + _fe(c)
    add = seg.get("add", [])
    b += struct.pack("<Q", len(add))
    for in0, out, c in add:
        b += struct.pack("<QQ", in0, out) + _fe(c)
    const = seg.get("const", [])
    b += struct.pack("<Q", len(const))
    for out, c in const:
        b += struct.pack("<Q", out) + _fe(c)
    rand = seg.get("rand", [])
    b += struct.pack("<Q", len(rand))
    for r in rand:
        b += struct.pack("<Q", r)
    return b


def circuit2_bytes(segments, layers, rand_sentinel=7):
    b = struct.pack("<QQ", MAGIC, len(segments))
    for s in segments:
        b += segment_bytes(s)
    b += struct.pack("<Q", len(layers))
    for l in layers:
        b += struct.pack("<Q", l)
    return b + _fe(rand_sentinel)


def random_circuit2(seed, depth=4, width=8, gadget=3):
    """A compiler-like CIRCUIT2 circuit: per layer a top segment of width 2^width whose gates
    come from a leaf gadget (2^gadget in and out, mixed mul/add/const gates, some with random
    coefficients) placed by a middle segment several times, which the top segment places
    again; one layer also holds direct gates.  Every flattened layer spans exactly 2^width
    inputs and outputs, so the layers chain."""
    st = gc.Stream(seed)
    segs = []
    layers = []
    g = 1 << gadget
    for d in range(depth):
        n = int(st.below(1, 2 * g)[0]) + g
        ins = st.below(3 * n, g).reshape(n, 3)
        kinds = st.below(n, 3)
        mul, add, const = [], [], []
        for k in range(n):
            c = int(st.u64(1)[0] & 0xFFFFFFFF)
            if kinds[k] == 0:
                mul.append((int(ins[k, 0]), int(ins[k, 1]), int(ins[k, 2]), c))
            elif kinds[k] == 1:
                add.append((int(ins[k, 0]), int(ins[k, 2]), c))
            else:
                const.append((int(ins[k, 2]), c))
        # the gadget's corners pin the layer's largest ids: input and output g - 1 are used
        mul.append((g - 1, 0, g - 1, 1))
        add.append((g - 1, g - 1, 1))
        rand = [0, len(mul)] if len(mul) > 1 else []
        leaf = len(segs)
        segs.append(dict(i_len=g, o_len=g, mul=mul, add=add, const=const, rand=rand))
        half = 1 << (width - 1)
        mid = len(segs)
        segs.append(dict(i_len=half, o_len=half, children=[(leaf, [(j * g, j * g) for j in range(half // g)])]))
        top = len(segs)
        extra = dict(mul=[(1, 2, 3, 5)], add=[(4, 5, 9)]) if d == 1 else {}
        segs.append(dict(i_len=2 * half, o_len=2 * half, children=[(mid, [(0, 0), (half, half)])], **extra))
        layers.append(top)
    return circuit2_bytes(segs, layers)


def extracted_text(circuit):
    """The two text files of Circuit::load_extracted_gates for `circuit` (line i holds layer
    L - 1 - i: mul "in0 in1 out coef", add "in0 out coef")."""
    ml, al = [], []
    for layer in reversed(circuit.layers):
        m = " ".join(f"{g[1]} {g[2]} {g[0]} {g[3]}" for g in layer.mul.tolist())
        a = " ".join(f"{g[1]} {g[0]} {g[2]}" for g in layer.add.tolist())
        ml.append(f"{layer.nb_mul_gates} {m}".rstrip())
        al.append(f"{layer.nb_add_gates} {a}".rstrip())
    return "\n".join(ml) + "\n", "\n".join(al) + "\n"


def sorted_gates(mul, add):
    mul = np.asarray(mul, np.uint32).reshape(-1, 4)
    add = np.asarray(add, np.uint32).reshape(-1, 3)
    mo = np.lexsort(mul.T[::-1]) if len(mul) else []
    ao = np.lexsort(add.T[::-1]) if len(add) else []
    return mul[mo], add[ao]
