"""The multi-GPU mode is replicas only: each rank proves its own proofs and the ranks meet
only at host barriers and a max over the timed regions.  This covers that plumbing
(bench.Dist) with two gloo ranks on the CPU."""
import os
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_two_rank_barrier_and_max(tmp_path):
    pytest.importorskip("torch")
    script = tmp_path / "ranks.py"
    script.write_text(textwrap.dedent(f"""
        import os, sys
        sys.path.insert(0, {ROOT!r})
        import bench
        d = bench.Dist()
        d.barrier()
        got = d.max(10.0 + d.rank)
        tot = d.sum(1.0)
        d.barrier()
        print("RANK", d.rank, d.world, got, tot, flush=True)
        d.close()
    """))
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT="29517", WORLD_SIZE="2")
    procs = []
    for r in range(2):
        e = dict(env, RANK=str(r), LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=e, stdout=subprocess.PIPE,
                                      stderr=subprocess.STDOUT, text=True))
    outs = [p.communicate(timeout=120)[0] for p in procs]
    for r, (p, o) in enumerate(zip(procs, outs)):
        assert p.returncode == 0, o
        assert f"RANK {r} 2 11.0 2.0" in o, o
