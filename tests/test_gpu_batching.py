"""GPU tests of continuous batching (several device lanes), the HBM budget, row tiles and
the autotuner.  Every proof must stay byte-identical to the reference golden whatever the
concurrency or tile: the tolerance is zero."""
import hashlib
import json
import os

import numpy as np
import pytest

import cases
from gkr_gb300 import circuit as gc

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["cases"]
MIX = ["cfg1_n16", "lanes1024", "mixed_widths_n16", "width_one_n8", "lanes48", "cfg1_n8", "lanes256",
       "local_wiring_n32", "all_mul_n16", "sparse_top_n32", "lanes4", "grind12_n16"]


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


@pytest.fixture()
def fresh_ctx():
    from gkr_gb300.prover import Context
    c = Context(0)
    yield c
    c.close()


def run_mix(ctx, names, repeat=1):
    built = [cases.build(n) for n in names]
    dcs = [ctx.load(c) for c, _, _ in built]
    jobs = []
    for _ in range(repeat):
        for name, (c, w, g), dc in zip(names, built, dcs):
            pb = np.empty(dc.proof_size(w.shape[1], g), np.uint8)
            cb = np.empty((3, w.shape[1]), np.uint32)
            jobs.append((name, ctx.submit(dc, w, pb, cb, grinding_bits=g), pb, cb))
    for name, job, pb, cb in jobs:
        n = ctx.wait(job)
        assert sha(pb[:n].tobytes()) == GOLDEN[name]["proof_sha256"], name
        assert sha(cb.tobytes()) == GOLDEN[name]["claimed_v_sha256"], name


def test_concurrent_lanes_byte_identical(fresh_ctx):
    fresh_ctx.set_concurrency(lanes=6)
    run_mix(fresh_ctx, MIX, repeat=3)
    fresh_ctx.set_concurrency(lanes=1)
    run_mix(fresh_ctx, MIX[:4])


def test_hbm_budget_bounds_the_workspaces(fresh_ctx):
    from gkr_gb300 import _lib
    lib = _lib.load()
    sizes = []
    for name in MIX:
        c, w, g = cases.build(name)
        dc = fresh_ctx.load(c)
        sizes.append(lib.gkrgpu_workspace_bytes(dc.handle, w.shape[1], g, 0))
    budget = max(sizes) + min(sizes)  # at most one large proof at a time
    fresh_ctx.set_concurrency(lanes=8, hbm_budget_bytes=budget)
    run_mix(fresh_ctx, MIX, repeat=2)
    st = fresh_ctx.memory_stats()
    assert st["budget"] == budget
    assert st["peak"] <= budget
    assert st["in_use"] == 0


@pytest.mark.parametrize("tile", [(8, 256, 0), (128, 256, 0), (32, 128, 152), (16, 256, 4864)])
def test_row_tiles_do_not_change_proofs(fresh_ctx, tile):
    fresh_ctx.set_tile(*tile)
    for name in ["cfg1_n16", "lanes1024", "lanes48", "width_one_n8"]:
        c, w, g = cases.build(name)
        cv, proof = fresh_ctx.prove(fresh_ctx.load(c), w, grinding_bits=g)
        assert sha(proof) == GOLDEN[name]["proof_sha256"], (name, tile)


def test_autotune_picks_tiles_and_keeps_bytes(fresh_ctx):
    circ = gc.random_circuit(31, [12, 13, 12, 13], p_mul=0.6, p_local=0.8, window=256)
    w = gc.random_witness(31, circ.log_input_size, 256)
    dc = fresh_ctx.load(circ)
    before = fresh_ctx.prove(dc, w)[1]
    choice = fresh_ctx.autotune(dc, w)
    for k in ["evaluate", "hg_build_round0", "round_fold_lane", "round_fold_scalar"]:
        assert choice[k]["threads_per_row"] in (8, 16, 32, 64)
        assert choice[k]["ms"] > 0
    after = fresh_ctx.prove(dc, w)[1]
    assert before == after
