"""Named, seeded parity cases shared by the golden-fixture generator and the tests.

Each case builds (circuit, witness, grinding_bits).  Lane counts are those the compiled
reference driver is instantiated for, so every case has a reference-generated golden.
"""
import numpy as np

from gkr_gb300 import circuit as gc


def _gkr_test_shape():
    # tests/GKR_Test.cpp:40-45: layers random(i+1, i+2) for i = 3..0 (deterministic wiring)
    return gc.Circuit([gc.CircuitLayer.random(i + 1, i + 2) for i in range(3, -1, -1)])


def _all_to_one(nb):
    # every gate reads input 0 and writes a handful of outputs; duplicate gates included
    layers = []
    for _ in range(3):
        O = 1 << nb
        o = np.arange(O, dtype=np.uint32)
        mul = np.stack([o, np.zeros(O, np.uint32), np.zeros(O, np.uint32), (o * 7 + 3) % gc.P], 1)
        mul = np.concatenate([mul, mul[:4]])  # duplicates
        add = np.stack([o // 2, np.zeros(O, np.uint32), np.ones(O, np.uint32)], 1)
        layers.append(gc.CircuitLayer(nb, nb, mul, add))
    return gc.Circuit(layers)


def _sparse_top(seed):
    # a wide input feeding a narrow layer (many x without gates), then an O = 1 output
    st = gc.Stream(seed)
    return gc.Circuit([gc.random_layer(st, 3, 6), gc.random_layer(st, 0, 3, p_mul=1.0)])


def _no_gates_layer():
    # a layer whose gates touch only half of the outputs; one layer with no add gates
    st = gc.Stream(77)
    l0 = gc.random_layer(st, 4, 4, p_mul=1.0)
    l1 = gc.random_layer(st, 4, 4, p_mul=0.0)
    l1.add = l1.add[: len(l1.add) // 2]
    return gc.Circuit([l0, l1])


CASES = {
    "cfg1_n8": lambda: (gc.config1_circuit(), 8, 10),
    "cfg1_n16": lambda: (gc.config1_circuit(), 16, 10),
    "gkr_test_shape_n8": lambda: (_gkr_test_shape(), 8, 10),
    "gkr_test_shape_n16": lambda: (_gkr_test_shape(), 16, 10),
    "mixed_widths_n16": lambda: (gc.random_circuit(5, [3, 2, 4, 1, 2]), 16, 10),
    "width_one_n8": lambda: (gc.random_circuit(6, [1, 1, 1, 1]), 8, 10),
    "output_scalar_n16": lambda: (gc.random_circuit(7, [3, 2, 0]), 16, 10),
    "all_add_n16": lambda: (gc.random_circuit(8, [5, 5, 5], p_mul=0.0), 16, 10),
    "all_mul_n16": lambda: (gc.random_circuit(9, [5, 5, 5], p_mul=1.0), 16, 10),
    "all_to_one_n8": lambda: (_all_to_one(4), 8, 10),
    "sparse_top_n32": lambda: (_sparse_top(10), 32, 10),
    "no_gates_rows_n16": lambda: (_no_gates_layer(), 16, 10),
    "lanes4": lambda: (gc.random_circuit(12, [6, 5, 6, 4]), 4, 10),
    "lanes48": lambda: (gc.random_circuit(13, [6, 5, 6, 4]), 48, 10),
    "lanes64": lambda: (gc.random_circuit(14, [7, 6, 7]), 64, 10),
    "lanes128": lambda: (gc.random_circuit(15, [6, 7, 5]), 128, 10),
    "lanes256": lambda: (gc.random_circuit(16, [5, 6, 4]), 256, 10),
    "lanes1024": lambda: (gc.random_circuit(17, [5, 4, 5]), 1024, 10),
    "local_wiring_n32": lambda: (gc.random_circuit(18, [8, 10, 8, 10, 8], p_mul=0.6, p_local=0.8, window=64), 32, 10),
    "grind8_n16": lambda: (gc.random_circuit(19, [4, 4, 4]), 16, 8),
    "grind12_n16": lambda: (gc.random_circuit(20, [4, 4, 4]), 16, 12),
}


# The benchmark's own circuits at copy counts the reference proves in seconds: the config-2
# proof (24 layers alternating 2^18 / 2^20 gates, 60% mul, window-local wiring) and, below,
# the config-4 BN254 proof (16 layers of 2^16 gates).  Their witness seeds are recorded in
# the golden file, so the benchmark can rebuild the same inputs without this module.
LARGE_CASES = {
    "cfg2_n8": lambda: (gc.config2_circuit(), 8, 10),
    "cfg2_n16": lambda: (gc.config2_circuit(), 16, 10),
}


def witness_seed(name):
    return sum(ord(c) for c in name) * 7919


def build(name):
    circ, n, grind = {**CASES, **LARGE_CASES}[name]()
    return circ, gc.random_witness(witness_seed(name), circ.log_input_size, n), grind


# ---------------------------------------------------------------- BN254 (Config::field_type = BN254)
def _full_range_coefs(circ, seed):
    # coefficients anywhere in [0, 2^32): canonical BN254 elements, most of them >= 2^31 - 1
    st = gc.Stream(seed)
    for l in circ.layers:
        if l.nb_mul_gates:
            l.mul[:, 3] = (st.u64(l.nb_mul_gates) >> np.uint64(32)).astype(np.uint32)
        if l.nb_add_gates:
            l.add[:, 2] = (st.u64(l.nb_add_gates) >> np.uint64(32)).astype(np.uint32)
    return circ


BN_CASES = {
    "bn_gkr_test_shape_n8": lambda: (_gkr_test_shape(), 8, 10),
    "bn_mixed_widths_n16": lambda: (gc.random_circuit(5, [3, 2, 4, 1, 2]), 16, 10),
    "bn_width_one_n4": lambda: (gc.random_circuit(6, [1, 1, 1, 1]), 4, 10),
    "bn_output_scalar_n16": lambda: (gc.random_circuit(7, [3, 2, 0]), 16, 10),
    "bn_full_coefs_n8": lambda: (_full_range_coefs(gc.random_circuit(21, [5, 4, 5]), 21), 8, 10),
    "bn_all_to_one_n4": lambda: (_all_to_one(4), 4, 10),
    "bn_no_gates_rows_n16": lambda: (_no_gates_layer(), 16, 10),
    "bn_lanes64": lambda: (gc.random_circuit(22, [6, 5, 6]), 64, 10),
    "bn_edge_values_n8": lambda: (gc.random_circuit(24, [4, 5, 4]), 8, 10),
    "bn_grind0_n8": lambda: (gc.random_circuit(23, [4, 4, 4]), 8, 0),
    "bn_grind12_n16": lambda: (gc.random_circuit(25, [4, 4, 4]), 16, 12),
}


BN_LARGE_CASES = {
    "bn_cfg4_n4": lambda: (gc.config4_circuit(), 4, 10),
    "bn_cfg4_n8": lambda: (gc.config4_circuit(), 8, 10),
}


def build_bn(name):
    """(circuit, (rows, N, 4) uint64 witness, grinding_bits) of a BN254 case."""
    circ, n, grind = {**BN_CASES, **BN_LARGE_CASES}[name]()
    w = gc.random_witness_bn254(witness_seed(name), circ.log_input_size, n)
    if name == "bn_edge_values_n8":
        r_minus_1 = [(gc.BN254_R - 1) >> (64 * k) & (2**64 - 1) for k in range(4)]
        w[0, :, :] = np.array(r_minus_1, np.uint64)  # r - 1 everywhere in row 0
        w[1, :, :] = 0  # zero row
        w[2, ::2, :] = np.array([1, 0, 0, 0], np.uint64)
        w[3, 1::2, :] = np.array(r_minus_1, np.uint64)
    return circ, w, grind
