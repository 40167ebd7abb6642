"""CPU tests of the circuit model and the seeded synthetic workloads."""
import numpy as np
import pytest

from gkr_gb300 import circuit as gc


def test_stream_is_pinned():
    # SplitMix64 of key 0 at counters 1, 2, 3: the workloads and golden fixtures depend on
    # this stream being identical on every machine.
    v = gc.Stream(0).u64(3)
    assert [int(x) for x in v] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
    s = gc.Stream(5)
    a = s.u64(4)
    b = s.u64(4)
    assert not np.array_equal(a, b)
    c = gc.Stream(5)
    assert np.array_equal(np.concatenate([c.u64(2), c.u64(6)]), np.concatenate([a, b]))


def test_field_samples_are_canonical():
    f = gc.Stream(1).field(100000)
    assert f.dtype == np.uint32 and int(f.max()) < gc.P


def test_config1_shape():
    c = gc.config1_circuit()
    c.validate()
    assert len(c.layers) == 8
    for l in c.layers:
        assert l.nb_input_vars == l.nb_output_vars == 10
        outs = np.concatenate([l.mul[:, 0], np.unique(l.add[:, 0])])
        assert len(np.unique(outs)) == 1024  # every output is exactly one gate
        assert l.nb_add_gates % 2 == 0


def test_config2_small_shape_and_locality():
    c = gc.random_circuit(3, [10, 12, 10], p_mul=0.6, p_local=0.8, window=64)
    c.validate()
    l = c.layers[0]
    O, I = 1 << l.nb_output_vars, 1 << l.nb_input_vars
    centre = (l.mul[:, 0].astype(np.int64) * I) // O
    local = (l.mul[:, 1] // 64) == (centre // 64)
    assert 0.75 < local.mean() < 0.9
    assert 0.55 < l.nb_mul_gates / O < 0.65


def test_validate_rejects_bad_circuits():
    c = gc.random_circuit(1, [3, 3])
    c.layers[0].mul[0, 1] = 8
    with pytest.raises(ValueError):
        c.validate()
    c = gc.random_circuit(1, [3, 3, 2])
    c.layers[1].nb_input_vars = 2
    with pytest.raises(ValueError):
        c.validate()
    c = gc.random_circuit(1, [3, 3])
    c.layers[0].add[0, 2] = gc.P
    with pytest.raises(ValueError):
        c.validate()


def test_proof_size_formula():
    c = gc.config1_circuit()
    # 80 416 bytes at 8 copies: the reference's proof for this shape
    assert c.proof_size(8) == 80416
    assert c.proof_size(16) == 160800
