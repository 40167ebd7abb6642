"""Circuit file loaders (gkrgpu_circuit2_parse, gkrgpu_extracted_parse) against the
reference's own loaders (CircuitRaw + Circuit::from_circuit_raw, load_extracted_gates),
compiled into oracle/_ref.  The parsers are host code and their tests run without a GPU;
the last test proves a loaded circuit on the GPU against the oracle."""
import struct

import numpy as np
import pytest

import circuit_files as cf
from gkr_gb300 import circuit as gc


@pytest.fixture(scope="module")
def lib():
    from gkr_gb300 import build as libbuild
    libbuild.build()
    from gkr_gb300 import _lib
    return _lib


def _same_layers(ours, theirs):
    assert len(ours.layers) == len(theirs)
    for k, (l, (nb_in, nb_out, mul, add)) in enumerate(zip(ours.layers, theirs)):
        assert (l.nb_input_vars, l.nb_output_vars) == (nb_in, nb_out), k
        m1, a1 = cf.sorted_gates(l.mul, l.add)
        m2, a2 = cf.sorted_gates(mul, add)
        assert np.array_equal(m1, m2), k
        assert np.array_equal(a1, a2), k


def _shared_leaf_file():
    # one gadget used by two layers, placed with overlapping outputs (duplicate output ids),
    # a const-only segment, and a largest id that is an exact power of two (the reference's
    # _compute_nb_vars then gives one bit less than the ids need)
    leaf = dict(i_len=4, o_len=4, mul=[(0, 1, 2, 3), (3, 3, 3, 4)], add=[(1, 0, 5)], const=[(2, 6)], rand=[1])
    consts = dict(i_len=2, o_len=2, const=[(0, 1), (1, 2)])
    top0 = dict(i_len=8, o_len=8, children=[(0, [(0, 0), (4, 4), (4, 0)]), (1, [(0, 0)])])
    top1 = dict(i_len=8, o_len=8, children=[(0, [(0, 0), (4, 4)])], add=[(0, 7, 1)])
    top2 = dict(i_len=16, o_len=16, mul=[(0, 16, 8, 1)])  # max id 16 = 2^4
    return cf.circuit2_bytes([leaf, consts, top0, top1, top2], [2, 3, 2, 4])


@pytest.mark.parametrize("seed,depth,width,gadget", [(1, 3, 6, 2), (2, 5, 8, 3), (3, 2, 10, 4)])
def test_circuit2_matches_reference_loader(lib, reference, seed, depth, width, gadget):
    data = cf.random_circuit2(seed, depth, width, gadget)
    ours = gc.Circuit.from_circuit2(data)
    _same_layers(ours, reference.circuit2_layers(data))
    # chained widths and coefficient 1 everywhere, as the reference loads it
    assert all(l.nb_input_vars == width and l.nb_output_vars == width for l in ours.layers)
    assert all((l.mul[:, 3] == 1).all() and (l.add[:, 2] == 1).all() for l in ours.layers)
    ours.validate()


def test_circuit2_shared_segments_and_quirks(lib, reference):
    data = _shared_leaf_file()
    ours = gc.Circuit.from_circuit2(data)
    _same_layers(ours, reference.circuit2_layers(data))
    # layer 3: largest id 16 -> next_pow_of_2(16) = 16 -> 4 variables, too few for id 16
    assert ours.layers[3].nb_input_vars == 4
    with pytest.raises(ValueError):
        ours.validate()


def test_extracted_text_matches_reference_loader(lib, reference, tmp_path):
    circ = gc.random_circuit(31, [5, 4, 6, 3])
    m, a = cf.extracted_text(circ)
    (tmp_path / "mul.txt").write_text(m)
    (tmp_path / "add.txt").write_text(a)
    ours = gc.Circuit.from_extracted(str(tmp_path / "mul.txt"), str(tmp_path / "add.txt"))
    _same_layers(ours, reference.extracted_layers(str(tmp_path / "mul.txt"), str(tmp_path / "add.txt")))
    # the wiring round-trips (sizes come from the largest ids, as in the reference)
    for l0, l1 in zip(circ.layers, ours.layers):
        assert np.array_equal(cf.sorted_gates(l0.mul, l0.add)[0], cf.sorted_gates(l1.mul, l1.add)[0])
    same = gc.Circuit.from_extracted(m, a)
    assert all(np.array_equal(x.mul, y.mul) for x, y in zip(ours.layers, same.layers))


@pytest.mark.parametrize("mutate,what", [
    (lambda b: b[:8], "truncated"),
    (lambda b: struct.pack("<Q", 1234) + b[8:], "magic"),
    (lambda b: b[:-40], "truncated"),
    (lambda b: b[:8] + struct.pack("<Q", 1 << 60) + b[16:], "count"),
])
def test_circuit2_malformed_files_are_rejected(lib, mutate, what):
    data = cf.random_circuit2(5, 2, 6, 2)
    with pytest.raises(lib.GkrGpuError) as e:
        gc.Circuit.from_circuit2(mutate(data))
    assert e.value.code == lib.ERR_INVALID


def test_circuit2_bad_references_are_rejected(lib):
    leaf = dict(i_len=2, o_len=2, mul=[(0, 1, 1, 1)])
    bad_child = dict(i_len=4, o_len=4, children=[(9, [(0, 0)])])
    cyc_a = dict(i_len=4, o_len=4, children=[(2, [(0, 0)])])
    cyc_b = dict(i_len=4, o_len=4, children=[(1, [(0, 0)])])
    bad_rand = dict(i_len=2, o_len=2, mul=[(0, 1, 1, 1)], rand=[5])
    for segs, layers in [([leaf, bad_child], [1]), ([leaf, cyc_a, cyc_b], [1]), ([leaf], [3]), ([bad_rand], [0])]:
        with pytest.raises(lib.GkrGpuError) as e:
            gc.Circuit.from_circuit2(cf.circuit2_bytes(segs, layers))
        assert e.value.code == lib.ERR_INVALID


def test_extracted_malformed_is_rejected(lib):
    with pytest.raises(lib.GkrGpuError):
        gc.Circuit.from_extracted("2 0 1 1 1\n", "1 0 0 1\n")  # two gates announced, one given
    with pytest.raises(lib.GkrGpuError):
        gc.Circuit.from_extracted("1 0 1 1 1\n1 0 0 0 1\n", "0\n")  # add file has fewer layers


@pytest.mark.gpu
@pytest.mark.parametrize("seed,depth,width,gadget,n", [(2, 5, 8, 3, 16), (3, 2, 10, 4, 64)])
def test_gpu_proves_loaded_circuit2(ctx, oracle, seed, depth, width, gadget, n):
    circ = gc.Circuit.from_circuit2(cf.random_circuit2(seed, depth, width, gadget))
    w = gc.random_witness(seed, circ.log_input_size, n)
    cv, proof = ctx.prove(ctx.load(circ), w)
    ocv, oproof = oracle.prove(circ, w)
    assert proof == oproof and np.array_equal(cv, ocv)
    assert oracle.verify(circ, w, cv, proof)
