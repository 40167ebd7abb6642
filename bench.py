#!/usr/bin/env python
"""Benchmark of the GB300 GKR prover on the large plain workload.

Workload (one step = one complete Prover::prove: RAW commitment, grinding, Circuit::evaluate
and the GKR sumcheck of every layer): a seeded synthetic M31 circuit of 24 layers whose
widths alternate 2^18 / 2^20 gates, 60% fan-in-2 mul / 40% fan-in-2 add, wiring local to
2^12-gate windows with probability 0.8, 1024 data-parallel copies, uniform witness,
SHA-256 transcript, RAW commitment.  The witness (1 GiB) and the per-layer tables
(~90 GiB) are far larger than L2, so no flush is needed between steps.

  value : proofs/s with the input already resident in HBM (gkrgpu_prove_submit with a
          device input), 6 proofs in flight so the host SHA-256 of the next proofs' RAW
          commitments overlaps the device work of the current ones, and two device lanes,
          so two proofs' device stages overlap (one proof's host round trips and
          integer-bound kernels leave HBM idle that the other proof's kernels use); timed
          from the device end of the last warm-up proof to the last device end among the
          timed proofs
  e2e   : the same through the C ABI from pinned host buffers (input H2D, claims and
          round rows D2H inside every step)
  roofline: the kernel with the largest device time; achieved = its algorithmic bytes per
          launch / its CUDA-event time per launch, against the measured HBM copy peak.
  cpu_baseline: the CPU oracle port (oracle/gkr_oracle.c) on this host's cores, one proof
          per thread, on the same circuit at 8 copies, scaled to 1024-copy proofs/s.

--impl reference runs the CPU prover alone (the compiled reference where it was built on
this machine, else the oracle port) and prints the same JSON line with "impl".
Multi-GPU (torchrun): independent replicas, one per rank, no data-path collective.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "expander-cpp_gb300")]

import numpy as np  # noqa: E402

METRIC = "GKR proofs/s batched vs plain on 1 GB300 (byte-identical proofs); p99; HBM GB/s"
UNIT = "proofs/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--copies", type=int, default=1024)
    ap.add_argument("--layers", type=int, default=24)
    ap.add_argument("--narrow", type=int, default=18)
    ap.add_argument("--wide", type=int, default=20)
    ap.add_argument("--cpu-copies", type=int, default=8, help="copies per proof in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--depth", type=int, default=6, help="proofs in flight (host hashing overlaps device work)")
    ap.add_argument("--tile", default="", help="threads_per_row,block,ctas for every kernel (default: autotuned)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the library's default row tiles")
    ap.add_argument("--workload", choices=["plain", "mixed", "serve", "bn254"], default="plain",
                    help="plain: the large single-circuit proof; mixed: many independent proofs of mixed depth, "
                         "width and copies, plain one-at-a-time vs continuous batching; serve: open-loop Poisson "
                         "arrivals of mixed proofs; bn254: 16 x 2^16 BN254 circuit at 64 copies, plain and "
                         "64 proofs batched")
    ap.add_argument("--proofs", type=int, default=512, help="mixed/serve: number of distinct proofs")
    ap.add_argument("--lanes", type=int, default=16, help="mixed/serve: proofs whose device stages overlap")
    ap.add_argument("--plain-lanes", type=int, default=2,
                    help="plain: proofs whose device stages overlap (one proof's per-round host round trips "
                         "and integer-bound kernels leave HBM idle unless another proof's kernels fill it)")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="mixed/serve: device-memory admission budget")
    ap.add_argument("--no-batched", action="store_true",
                    help="plain: no mixed batched-vs-plain object; bn254: only the plain proofs (no 64-proof batch)")
    ap.add_argument("--batched-proofs", type=int, default=128,
                    help="plain: proofs of the shortened mixed workload measured batched and one at a time")
    ap.add_argument("--no-keccak", action="store_true", help="plain: skip the Keccak-256 transcript rate")
    ap.add_argument("--no-parity", action="store_true", help="plain: skip the golden and verifier checks")
    ap.add_argument("--no-round-tail", action="store_true",
                    help="plain: every sumcheck round as its own launch (no persistent phase tails)")
    ap.add_argument("--rates", default="200,500,1000,2000", help="serve: arrival rates (requests/s)")
    ap.add_argument("--duration", type=float, default=4.0, help="serve: seconds of arrivals per rate")
    ap.add_argument("--serve-size", choices=["mixed", "config2"], default="mixed",
                    help="serve: request sizes (the mixed proofs, or the large config-2 proof)")
    ap.add_argument("--max-queue", type=int, default=512,
                    help="serve: requests waiting for admission beyond which new ones are rejected")
    ap.add_argument("--host-threads", type=int, default=0,
                    help="host threads for the commitment hashes (0: the library default)")
    return ap.parse_args()


# ---------------------------------------------------------------- distributed plumbing
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- workload
def workload(args):
    from gkr_gb300 import circuit as gc
    widths = [args.narrow if l % 2 == 0 else args.wide for l in range(args.layers + 1)]
    circ = gc.random_circuit(2024, widths, p_mul=0.6, p_local=0.8, window=1 << 12)
    cfg = {"workload": f"{args.layers} layers alternating 2^{args.narrow}/2^{args.wide} gates, 60% mul / 40% add "
                       f"fan-in-2, wiring local to 2^12-gate windows w.p. 0.8, {args.copies} copies, uniform M31 "
                       "witness, SHA-256 transcript, RAW commitment (one plain proof per step)",
           "n_copies": args.copies, "layers": args.layers, "widths_log2": [args.narrow, args.wide],
           "mul_gates": circ.nb_mul_gates, "add_gates": circ.nb_add_gates, "grinding_bits": 10, "repetitions": 3,
           "l2": "inputs and tables larger than L2 (no flush needed)", "field": "M31"}
    return circ, widths, cfg


def reference_formula_bytes(circ, n_copies, elem_bytes=4, reps=3):
    """Algorithmic bytes of one proof by the streaming model of the survey of the reference's
    path: per layer (2 Gm + Ga + O) vectors for evaluate, (Gm + R I) for the phase-one hg build,
    (1 + 5R) I for the phase-one rounds and (1 + 2R) I for phase two, plus the gate lists and
    scalar tables.  It counts traffic this prover does not move (hg tables never written, folded
    copies refolded instead of stored, rows without gates skipped), so a rate against it is an
    equivalent rate and can exceed the copy peak."""
    vec = elem_bytes * n_copies
    total, scalars = 0.0, 0.0
    for l in circ.layers:
        I, O = 1 << l.nb_input_vars, 1 << l.nb_output_vars
        gm = 0 if l.mul is None else len(l.mul)
        ga = 0 if l.add is None else len(l.add)
        total += (2 * gm + ga + O) + (gm + reps * I) + (1 + 5 * reps) * I + (1 + 2 * reps) * I
        scalars += 48 * gm + 24 * ga + 4 * reps * (2 * O + 2 * I)
    total += 1 << circ.layers[-1].nb_output_vars
    return vec * total + scalars


def cpu_sample(circ, args, n_steps=1, warmup=0):
    """Times the CPU prover (all host cores, one proof per thread) on the workload's circuit at
    args.cpu_copies copies.  Returns (per-step values scaled to args.copies-copy proofs/s,
    per-step measured seconds, info)."""
    from gkr_gb300 import circuit as gc
    from oracle.oracle import Oracle, Reference
    threads = len(os.sched_getaffinity(0))
    w = gc.random_witness(7, circ.log_input_size, args.cpu_copies)
    use_ref = Reference.available()
    if use_ref:
        ref = Reference()

        def run():
            t0 = time.perf_counter()
            ths = [threading.Thread(target=ref.prove, args=(circ, w), kwargs={"native": args.cpu_copies == 8})
                   for _ in range(threads)]
            for t in ths:
                t.start()
            for t in ths:
                t.join()
            return time.perf_counter() - t0
        kind = "reference"
    else:
        orc = Oracle()

        def run():
            return orc.bench(circ, w, threads, 1)
        kind = "port"
    for _ in range(warmup):
        run()
    vals, secs = [], []
    for _ in range(n_steps):
        dt = run()
        secs.append(dt)
        vals.append(threads / dt * args.cpu_copies / args.copies)
    info = {"cores": threads, "kind": kind,
            "sample": f"{threads} threads x 1 proof of the same circuit at {args.cpu_copies} copies (evaluate + prove, "
                      f"{statistics.mean(secs):.2f} s per sample), reported as {args.copies}-copy proofs/s: "
                      f"{threads} proofs x {args.cpu_copies}/{args.copies} per sample time",
            "sample_seconds": secs}
    if kind == "port":
        info["port_vs_reference"] = PORT_VS_REFERENCE
    return vals, secs, info


# The oracle port against the compiled reference (VectorizedM31, AVX-512) on the same
# 8-copy proof of this circuit, one thread each, measured on an x86-64 host where both
# build; the Arm GPU host has no reference tree, so there the port stands in for it.
PORT_VS_REFERENCE = {"port_s": 8.9, "reference_s": 6.1, "ratio": 1.45,
                     "note": "single-thread 8-copy config-2 proof on a Xeon with AVX-512; the port understates the "
                             "reference's CPU speed by about this factor"}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------- arms
def run_reference(args, D):
    if D.rank != 0:
        return
    circ, widths, cfg = workload(args)
    vals, secs, info = cpu_sample(circ, args, n_steps=args.steps, warmup=args.warmup)
    v = statistics.mean(vals)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * statistics.mean(secs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic", "config": cfg,
            "impl": "reference",
            "value_kind": f"scaled sample: each step proves {info['cores']} proofs at {args.cpu_copies} copies on "
                          f"{info['cores']} threads; value = {info['cores']} x {args.cpu_copies}/{args.copies} / "
                          "step seconds; ms_per_step is the measured step time",
            "cpu_baseline": dict(info, value=v, unit=UNIT),
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# Timing-marker slots (gkrgpu_elapsed_ms): proofs submitted with marker k record their
# device-stage end in slot k and its beginning in slot 64 + k; slot 63 is the reference
# mark taken before any proof of a pipelined run is submitted.
REF_SLOT = 63
MAX_TIMED = 62


def pipelined(ctx, n_warm, n_timed, bufs, submit):
    """Runs n_warm + n_timed proofs keeping len(bufs) in flight (host stage of the next
    proofs overlapping the device stage of the current ones).  The timed region runs from
    the earliest device-stage beginning among the timed proofs to the latest device-stage
    end among them, so it holds the whole device stage of every timed proof (and possibly
    the tail of a warm-up proof on another lane, which is not counted).  Returns (total ms,
    intervals between consecutive timed proof ends starting at the region's start,
    per-proof submit-to-done latency ms, kernel stats when the last warm-up proof and the
    last proof were waited for, per-proof device-stage ms)."""
    if n_timed > MAX_TIMED:
        raise ValueError(f"at most {MAX_TIMED} timed proofs per run")
    depth = len(bufs)
    total = n_warm + n_timed
    jobs, t_sub, lat = {}, {}, []
    stats0 = None
    ctx.mark(REF_SLOT)

    def sub(i):
        marker = i - n_warm if i >= n_warm else -1
        t_sub[i] = time.perf_counter()
        jobs[i] = submit(bufs[i % depth], marker)

    try:
        for i in range(min(depth, total)):
            sub(i)
        for i in range(total):
            ctx.wait(jobs.pop(i))
            lat.append((i, (time.perf_counter() - t_sub[i]) * 1000.0))
            if i == n_warm - 1:
                stats0 = ctx.kernel_stats()
            if i + depth < total:
                sub(i + depth)
    except BaseException:
        # the proofs still in flight write into these buffers: wait for them before unwinding
        for j in jobs.values():
            try:
                ctx.wait(j)
            except Exception:
                pass
        raise
    if stats0 is None:
        stats0 = {k: {"launches": 0, "ms": 0.0, "bytes": 0.0} for k in ctx.kernel_stats()}
    stats1 = ctx.kernel_stats()
    begins = [ctx.elapsed_ms(REF_SLOT, 64 + k) for k in range(n_timed)]
    ends = [ctx.elapsed_ms(REF_SLOT, k) for k in range(n_timed)]
    t0, t1 = min(begins), max(ends)
    e = sorted(ends)
    steps = [b - a for a, b in zip([t0] + e[:-1], e)]
    stage = [b - a for a, b in zip(begins, ends)]
    return t1 - t0, steps, [l for i, l in lat if i >= n_warm], stats0, stats1, stage


def stats_delta(s0, s1):
    return {k: {f: s1[k][f] - s0[k][f] for f in ("launches", "ms", "bytes")} for k in s1}


def kernel_table(stats, n_steps, traffic_ratios):
    """Per kernel kind: launches and device ms per step, the algorithmic-byte rate, and the
    DRAM rate (algorithmic bytes x the ncu DRAM/algorithmic ratio of that kind, where one was
    captured: gathers that hit L2 count as algorithmic bytes but not as DRAM traffic)."""
    out = {}
    for k, v in stats.items():
        if not v["launches"]:
            continue
        alg = (v["bytes"] / (v["ms"] / 1000.0) / 1e9) if v["ms"] and k not in NOT_BANDWIDTH else None
        r = traffic_ratios.get(k, {}).get("traffic_over_algorithmic")
        out[k] = {"launches_per_step": v["launches"] / n_steps, "ms_per_step": v["ms"] / n_steps,
                  "algorithmic_GBps": alg, "dram_GBps": alg * r if (alg and r) else None}
    return out


# Kinds whose event time is not their own work: a phase tail's launch spans the host round
# trips of its rounds (it waits for each challenge on the device).
NOT_BANDWIDTH = {"round_tail"}


def roofline_of(stats, traffic_ratios):
    """Roofline line of the kernel kind with the largest device time: its algorithmic bytes
    per launch over its CUDA-event time per launch, against the measured HBM copy peak."""
    peak, peak_kind = peaks()
    name, s = max(((k, v) for k, v in stats.items() if k not in NOT_BANDWIDTH), key=lambda kv: kv[1]["ms"])
    per_launch_bytes = s["bytes"] / max(s["launches"], 1)
    per_launch_ms = s["ms"] / max(s["launches"], 1)
    achieved = per_launch_bytes / (per_launch_ms / 1000.0) / 1e9 if per_launch_ms > 0 else 0.0
    ratio = traffic_ratios.get(name, {}).get("traffic_over_algorithmic")
    return {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": per_launch_bytes * ratio if ratio else None,
            "peak_source": peak_kind, "algorithmic_bytes_per_launch": per_launch_bytes, "launches": s["launches"],
            "ms_per_launch": per_launch_ms}


def load_traffic_ratios():
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    return json.load(open(tfile)) if os.path.exists(tfile) else {}


def golden_parity(ctx, dc, circ, name="cfg2_n8"):
    """Proves the benchmark circuit at the few copies of a golden case made by the compiled
    reference (tests/golden/golden.json) and compares the digests of the proof and claims."""
    import hashlib

    from gkr_gb300 import circuit as gc
    gfile = os.path.join(ROOT, "tests", "golden", "golden.json")
    g = json.load(open(gfile)).get("large_cases", {}).get(name) if os.path.exists(gfile) else None
    if g is None:
        return {"case": name, "result": "no golden"}
    w = gc.random_witness(g["witness_seed"], circ.log_input_size, g["n_copies"])
    cv, proof = ctx.prove(dc, w, grinding_bits=g["grinding_bits"])
    ok_p = hashlib.sha256(proof).hexdigest() == g["proof_sha256"] and len(proof) == g["proof_len"]
    ok_c = hashlib.sha256(np.ascontiguousarray(cv).tobytes()).hexdigest() == g["claimed_v_sha256"]
    return {"case": name, "n_copies": g["n_copies"], "proof_bytes": len(proof),
            "result": "golden" if (ok_p and ok_c) else "MISMATCH",
            "source": "digests of the compiled reference's proof of the same circuit and witness"}


def run_ours(args, D):
    from gkr_gb300 import circuit as gc
    from gkr_gb300.prover import Context, DeviceBuffer, HostBuffer

    if args.steps > MAX_TIMED:
        raise SystemExit(f"--steps must be <= {MAX_TIMED}")
    device = D.local_rank
    circ, widths, cfg = workload(args)
    N = args.copies
    ctx = Context(device)
    if args.host_threads:
        ctx.set_host_threads(args.host_threads)
    if args.no_round_tail:
        ctx.set_round_tail(False)
    if args.plain_lanes > 1:
        ctx.set_concurrency(lanes=args.plain_lanes)
    if args.tile:
        ctx.set_tile(*[int(x) for x in args.tile.split(",")])
    dc = ctx.load(circ)
    rows = 1 << circ.log_input_size
    plen = dc.proof_size(N)
    hin = HostBuffer(rows * N * 4, np.uint32)
    witness = hin.array.reshape(rows, N)
    gc.random_witness(1000 + D.rank, circ.log_input_size, N, out=witness)
    din = DeviceBuffer(ctx, rows * N * 4)
    din.upload(witness)
    depth = args.depth
    pbufs = [HostBuffer(plen) for _ in range(depth)]
    bufs = [(pb.array, np.empty((3, N), np.uint32)) for pb in pbufs]
    traffic = load_traffic_ratios()

    # row tiles from the autotuner (whole proofs timed per candidate; outside the timed region)
    tiles = None
    if not args.tile and not args.no_autotune:
        t0 = time.perf_counter()
        tiles = ctx.autotune(dc, None, n_copies=N, d_input=din.ptr)
        tiles = {"seconds": time.perf_counter() - t0,
                 "choice": {k: {"threads_per_row": v["threads_per_row"], "ctas": v["ctas"]}
                            for k, v in tiles.items() if v["ms"] > 0}}
        ctx.reset_stats()

    def dev_submit(b, m):
        return ctx.submit(dc, None, b[0], b[1], d_input=din.ptr, marker=m)

    # ---- value: input resident in HBM.  Per-launch CUDA events are kept only with one lane:
    # with two, another proof's kernels share the GPU and a launch's time is not its own
    one_lane = args.plain_lanes <= 1
    ctx.set_timing(one_lane)
    clocks = ClockSampler(device)
    clocks.start()
    D.barrier()
    total_ms, step_ms, lat_ms, s0, s1, stage_ms = pipelined(ctx, args.warmup, args.steps, bufs, dev_submit)
    D.barrier()
    clk = clocks.stop()
    ctx.set_timing(False)
    stats, stat_steps = stats_delta(s0, s1), args.steps
    max_ms = D.max(total_ms)
    value = D.world * args.steps / (max_ms / 1000.0)
    tail = [bytes(b[0][plen - 4096:plen]) for b in bufs[:min(depth, args.warmup + args.steps)]]
    assert all(t == tail[0] for t in tail), "proofs of the same input differ"

    # ---- e2e: host buffers through the C ABI (input H2D, claims and round rows D2H)
    e2e = None
    if not args.no_e2e:
        h0 = ctx.transfer_stats()
        D.barrier()
        e2e_warm = max(1, args.warmup)
        e2e_ms, e2e_steps, e2e_lat, _, _, _ = pipelined(
            ctx, e2e_warm, args.steps, bufs, lambda b, m: ctx.submit(dc, witness, b[0], b[1], marker=m))
        e2e_ms = D.max(e2e_ms)
        h1 = ctx.transfer_stats()
        n_jobs = e2e_warm + args.steps
        e2e = {"value": D.world * args.steps / (e2e_ms / 1000.0), "unit": UNIT,
               "h2d_bytes_per_step": (h1[0] - h0[0]) // n_jobs, "d2h_bytes_per_step": (h1[1] - h0[1]) // n_jobs,
               "ms_per_step": e2e_ms / args.steps,
               "latency_ms": {"p50": statistics.median(e2e_lat), "p99": float(np.percentile(e2e_lat, 99))},
               "note": f"gkrgpu_prove_submit/wait from pinned host memory, {depth} proofs in flight; the RAW "
                       "commitment is copied and hashed on the host from the input"}
        assert bytes(bufs[0][0][plen - 4096:plen]) == tail[0], "e2e proof differs from the device-input proof"

    # ---- the plain prover with one device lane (one proof's device stage at a time), then a
    # short one-lane pass with per-launch CUDA events for the kernel table and roofline
    plain1 = None
    kernel_timing = "per-launch CUDA events on the library's stream inside the timed region"
    if not one_lane:
        ctx.set_concurrency(lanes=1)
        n1 = min(args.steps, 12)
        p1_ms, _, p1_lat, _, _, p1_stage = pipelined(ctx, 2, n1, bufs[:4], dev_submit)
        plain1 = {"proofs_per_s": n1 / (p1_ms / 1000.0), "ms_per_proof": p1_ms / n1, "steps": n1,
                  "device_stage_ms_median": statistics.median(p1_stage),
                  "note": "one device lane, 4 proofs in flight (host stages of the next proofs overlap), "
                          "device input"}
        ctx.set_timing(True)
        kp_steps = 2
        _, _, _, k0, k1, _ = pipelined(ctx, 1, kp_steps, bufs, dev_submit)
        ctx.set_timing(False)
        stats, stat_steps = stats_delta(k0, k1), kp_steps
        kernel_timing = (f"per-launch CUDA events in a one-lane pass of {kp_steps} proofs after the timed regions "
                         f"(with {args.plain_lanes} lanes another proof's kernels share the GPU, so a launch's time "
                         "there is not its own)")
        ctx.set_concurrency(lanes=args.plain_lanes)
    launches_per_proof = sum(s["launches"] for s in stats.values()) / stat_steps
    launches = int(round(launches_per_proof * args.steps))

    # ---- parity of the timed circuit: the golden of the compiled reference at 8 copies, and
    # the library's verifier (Verifier::verify) on one timed 1024-copy proof
    parity = None
    if not args.no_parity and D.rank == 0:
        parity = golden_parity(ctx, dc, circ)
        t0 = time.perf_counter()
        ok = ctx.verify(dc, bufs[0][0][:plen], bufs[0][1])
        parity["timed_proof_verified"] = bool(ok)
        parity["verify_s"] = time.perf_counter() - t0

    # ---- the same proofs with the Keccak-256 transcript (host hashing of the commitment,
    # challenges and grinding with Keccak-f[1600] instead of SHA-256)
    keccak = None
    if not args.no_keccak:
        # the Keccak-256 of a 1 GiB commitment runs about three times longer than its SHA-256
        # (portable code on the host): twice the host threads keep the host stages ahead
        ctx.set_fs_hash("Keccak256")
        ctx.set_host_threads(8)
        nk = min(args.steps, 8)
        k_ms, _, k_lat, _, _, _ = pipelined(ctx, 2, nk, bufs, dev_submit)
        ktail = [bytes(b[0][plen - 4096:plen]) for b in bufs[:min(depth, nk + 2)]]
        ctx.set_host_threads(args.host_threads)
        ctx.set_fs_hash("SHA256")
        keccak = {"proofs_per_s": nk / (k_ms / 1000.0), "ms_per_proof": k_ms / nk, "steps": nk,
                  "consistent": all(t == ktail[0] for t in ktail) and ktail[0] != tail[0],
                  "note": f"Keccak-256 transcript, {args.plain_lanes} device lanes, {depth} in flight, 8 host threads, "
                          "device input"}

    roofline = roofline_of(stats, traffic)
    total_bytes = sum(v["bytes"] for v in stats.values()) / stat_steps
    ref_bytes = reference_formula_bytes(circ, N)
    kernel_ms = sum(v["ms"] for v in stats.values()) / stat_steps
    kernels = kernel_table(stats, stat_steps, traffic)
    din.free()
    ctx.close()

    # ---- batched vs plain on a shortened mixed workload (the metric's own comparison)
    batched = None
    if not args.no_batched and D.rank == 0:
        batched = measure_mixed(device, args.batched_proofs, args.lanes, int(args.budget_gb * (1 << 30)),
                                host_threads=args.host_threads)

    cpu = None
    if D.rank == 0 and not args.no_cpu_baseline:
        vals, _, info = cpu_sample(circ, args)
        cpu = dict(info, value=vals[0], unit=UNIT)

    if D.rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": D.world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
                "config": dict(cfg, parallelism=f"replicas x{D.world}" if D.world > 1 else "single",
                               pipeline=f"{depth} proofs in flight, {args.plain_lanes} device lane(s) (that many "
                                        "proofs' device stages overlap); timed region = earliest device-stage "
                                        "beginning to latest device-stage end among the timed proofs"),
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "autotune": tiles,
                "clocks": clk, "parity": parity, "plain_one_lane": plain1, "keccak": keccak, "batched": batched,
                "latency_ms": {"p50": statistics.median(lat_ms), "p99": float(np.percentile(lat_ms, 99)),
                               "device_end_intervals_ms": step_ms,
                               "device_stage_ms_median": statistics.median(stage_ms)},
                "hbm": {"algorithmic_bytes_per_proof": total_bytes,
                        "GBps_over_step": total_bytes / (max_ms / args.steps / 1000.0) / 1e9,
                        "GBps_over_kernels": total_bytes / (kernel_ms / 1000.0) / 1e9,
                        "kernel_ms_per_step": kernel_ms,
                        "reference_formula": {
                            "bytes_per_proof": ref_bytes,
                            "equivalent_GBps_over_step": ref_bytes / (max_ms / args.steps / 1000.0) / 1e9,
                            "note": "streaming-model bytes of the reference's path (evaluate, hg build, both "
                                    "phases' rounds, gate lists); counts traffic this prover avoids, so the "
                                    "equivalent rate can exceed the copy peak"}},
                "kernels": kernels, "kernel_timing": kernel_timing, "proof_bytes": plen}
        print(json.dumps(line), flush=True)


class MixedSet:
    """The mixed workload: independent proofs of uniform depth 4..24, width 2^8..2^18 and
    16..256 copies (multiples of 16), 50% mul / 50% add fan-in-2 gates with uniform wiring,
    each with its own seed; circuits resident on the device, witnesses in host memory."""

    def __init__(self, ctx, n_proofs, seed=3):
        from concurrent.futures import ThreadPoolExecutor

        from gkr_gb300 import circuit as gc
        self.specs = gc.mixed_batch_specs(seed=seed, n_proofs=n_proofs)
        with ThreadPoolExecutor(8) as ex:
            self.circuits = list(ex.map(lambda s: gc.uniform_circuit(s[0], s[1], s[2]), self.specs))
            self.witness = list(ex.map(lambda s: gc.random_witness(s[0], s[2], s[3]), self.specs))
        self.dcs = [ctx.load(c) for c in self.circuits]
        self.proofs = [np.empty(dc.proof_size(s[3]), np.uint8) for dc, s in zip(self.dcs, self.specs)]
        self.claims = [np.empty((3, s[3]), np.uint32) for s in self.specs]
        self.bytes = sum(s[1] * (1 << s[2]) * s[3] * 4 for s in self.specs)

    def submit(self, ctx, i):
        return ctx.submit(self.dcs[i], self.witness[i], self.proofs[i], self.claims[i])

    def digests(self, idx):
        import hashlib
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(8) as ex:
            return list(ex.map(lambda i: hashlib.sha256(self.proofs[i].tobytes()).hexdigest(), idx))


def measure_mixed(device, n_proofs, lanes, budget, seed=3, host_threads=0):
    """Plain (one proof at a time, one device lane) vs continuous batching (every proof
    queued at once, up to `lanes` device stages overlapping under the HBM budget) on the
    same independent mixed proofs; both modes' proofs are compared byte for byte."""
    from gkr_gb300.prover import Context
    ctx = Context(device)
    if host_threads:
        ctx.set_host_threads(host_threads)
    t0 = time.perf_counter()
    ms = MixedSet(ctx, n_proofs, seed=seed)
    setup_s = time.perf_counter() - t0
    n = len(ms.specs)
    idx = list(range(n))

    # plain: each proof submitted after the previous one finished (the reference's
    # one-proof-per-call usage, on the GPU)
    ctx.set_concurrency(lanes=1)
    for i in range(min(4, n)):
        ctx.wait(ms.submit(ctx, i))
    lat_plain = []
    t0 = time.perf_counter()
    for i in idx:
        t1 = time.perf_counter()
        ctx.wait(ms.submit(ctx, i))
        lat_plain.append((time.perf_counter() - t1) * 1000.0)
    plain_s = time.perf_counter() - t0
    ref = ms.digests(idx)

    ctx.set_concurrency(lanes=lanes, hbm_budget_bytes=budget)
    warm = [ms.submit(ctx, i) for i in range(min(2 * lanes, n))]
    for j in warm:
        ctx.wait(j)

    def one_batch():
        t0 = time.perf_counter()
        sub, jobs = {}, []
        for i in idx:
            sub[i] = time.perf_counter()
            jobs.append(ms.submit(ctx, i))
        done = []
        for i, j in zip(idx, jobs):
            ctx.wait(j)
            done.append((time.perf_counter() - sub[i]) * 1000.0)
        return time.perf_counter() - t0, done

    # the same batch with every round as its own launch (no persistent phase tails)
    ctx.set_round_tail(False)
    notail_s, _ = one_batch()
    same_notail = ms.digests(idx) == ref
    ctx.set_round_tail(True)
    clocks = ClockSampler(device)
    clocks.start()
    batch_s, done = one_batch()
    clk = clocks.stop()
    same = ms.digests(idx) == ref and same_notail
    mem = ctx.memory_stats()
    out = {"workload": f"{n} independent proofs, depth 4..24, width 2^8..2^18, 16..256 copies, 50% mul uniform "
                       "wiring, own seed each", "proofs": n, "lanes": lanes, "hbm_budget_bytes": budget,
           "setup_s": setup_s, "witness_bytes_total": ms.bytes,
           "timing": "host wall clock from the first submit to the last proof returned",
           "batched": {"proofs_per_s": n / batch_s, "seconds": batch_s,
                       "latency_ms": {"p50": statistics.median(done), "p99": float(np.percentile(done, 99))}},
           "plain": {"proofs_per_s": n / plain_s, "seconds": plain_s,
                     "latency_ms": {"p50": statistics.median(lat_plain), "p99": float(np.percentile(lat_plain, 99))}},
           "batched_over_plain": plain_s / batch_s, "byte_identical_to_plain": same,
           "batched_per_round_launches": {"proofs_per_s": n / notail_s, "seconds": notail_s,
                                          "note": "the same batch with the persistent phase tails off: every "
                                                  "sumcheck round its own kernel launch"},
           "host_threads": host_threads or "default",
           "hbm": {"workspace_peak_bytes": mem["peak"], "budget": mem["budget"]}, "clocks": clk}
    ctx.close()
    return out


def run_mixed(args, D):
    """Plain (one proof at a time) vs continuous batching on the same independent proofs."""
    if D.rank != 0:
        return
    r = measure_mixed(D.local_rank, args.proofs, args.lanes, int(args.budget_gb * (1 << 30)),
                      host_threads=args.host_threads)
    n = r["proofs"]
    line = {"metric": METRIC, "value": r["batched"]["proofs_per_s"], "unit": UNIT, "n_gpus": 1, "steps": n,
            "warmup": min(2 * args.lanes, n), "ms_per_step": r["batched"]["seconds"] * 1000.0 / n,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": r["workload"] + " (one batch)", "lanes": args.lanes,
                       "hbm_budget_bytes": r["hbm_budget_bytes"], "setup_s": r["setup_s"],
                       "witness_bytes_total": r["witness_bytes_total"], "timing": r["timing"]},
            "batched": r["batched"], "plain": r["plain"], "batched_over_plain": r["batched_over_plain"],
            "byte_identical_to_plain": r["byte_identical_to_plain"], "hbm": r["hbm"], "clocks": r["clocks"]}
    print(json.dumps(line), flush=True)


def serve_rate(srv, dcs, wits, rate, duration, seed):
    """One open-loop Poisson stream through the server: request r proves proof (r mod n);
    returns offered / admitted / rejected counts, completed proofs/s and p50 / p99 latency
    of the completed requests (arrival to proof returned)."""
    from gkr_gb300.serving import Rejected
    n = len(dcs)
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * duration * 1.5) + 8))
    arrivals = arrivals[arrivals < duration]
    futs = []
    t0 = time.perf_counter()
    for r, a in enumerate(arrivals):
        now = time.perf_counter() - t0
        if a > now:
            time.sleep(a - now)
        futs.append(srv.submit(dcs[r % n], wits[r % n]))
    lats, rejected = [], 0
    t_last = t0
    for f in futs:
        try:
            res = f.result()
            lats.append(res.latency_ms)
            res.release()
            t_last = max(t_last, time.perf_counter())
        except Rejected:
            rejected += 1
    wall = t_last - t0
    return {"offered": len(arrivals), "offered_per_s": len(arrivals) / duration, "admitted": len(lats),
            "rejected": rejected, "completed_per_s": len(lats) / wall if wall > 0 else None,
            "latency_ms": {"p50": statistics.median(lats), "p99": float(np.percentile(lats, 99))} if lats else None}


def run_serve(args, D):
    """Open-loop Poisson arrivals through the serving loop (gkr_gb300.serving.ProofServer):
    continuous batching over several device lanes vs one proof at a time (one lane), at each
    rate.  --serve-size mixed: the mixed proofs (depth 4..24, width 2^8..2^18, 16..256
    copies); config2: the large proof (two distinct 1 GiB witnesses; one proof's workspace
    fills most of the budget, so the server runs saturated and its bounded admission queue
    rejects the rest).  Witnesses are uploaded once per request at admission and stay
    resident until the proof is done; the proof reads the resident copy."""
    from gkr_gb300 import circuit as gc
    from gkr_gb300.prover import Context
    from gkr_gb300.serving import ProofServer
    if D.rank != 0:
        return
    ctx = Context(D.local_rank)
    if args.host_threads:
        ctx.set_host_threads(args.host_threads)
    budget = int(args.budget_gb * (1 << 30))
    if args.serve_size == "config2":
        circ = gc.config2_circuit()
        dc = ctx.load(circ)
        wits = [gc.random_witness(2000 + i, circ.log_input_size, 1024) for i in range(2)]
        dcs = [dc] * len(wits)
        desc = ("open-loop Poisson arrivals of the config-2 proof (24 layers 2^18/2^20, 1024 copies, "
                "2 distinct witnesses)")
        arena, max_queue, lanes = 4 << 30, 4, args.plain_lanes
    else:
        ms = MixedSet(ctx, args.proofs, seed=5)
        dcs, wits = ms.dcs, ms.witness
        desc = (f"open-loop Poisson arrivals over {len(dcs)} distinct mixed proofs (depth 4..24, width 2^8..2^18, "
                "16..256 copies)")
        arena, max_queue, lanes = 16 << 30, args.max_queue, args.lanes
    out = {}
    clocks = ClockSampler(D.local_rank)
    clocks.start()
    for mode, nl in (("batched", lanes), ("plain", 1)):
        srv = ProofServer(ctx, lanes=nl, budget_bytes=budget, arena_bytes=arena, max_queue=max_queue)
        for i in range(min(2 * nl, len(dcs))):  # warm-up
            srv.submit(dcs[i], wits[i]).result()
        res = {}
        for rate in [float(r) for r in args.rates.split(",")]:
            res[str(int(rate))] = serve_rate(srv, dcs, wits, rate, args.duration, int(rate))
        res["server"] = srv.stats()
        srv.close()
        out[mode] = dict(res, lanes=nl)
    clk = clocks.stop()
    top = out["batched"][str(int(float(args.rates.split(",")[-1])))]
    line = {"metric": METRIC, "value": top["completed_per_s"], "unit": UNIT, "n_gpus": 1,
            "steps": top["admitted"], "warmup": 2 * out["batched"]["lanes"],
            "ms_per_step": 1000.0 / top["completed_per_s"] if top["completed_per_s"] else None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": desc, "rates": args.rates, "duration_s": args.duration, "hbm_budget_bytes": budget,
                       "arena_bytes": arena, "max_queue": max_queue,
                       "timing": "host wall clock; latency = arrival to proof returned"},
            "serving": out, "clocks": clk}
    print(json.dumps(line), flush=True)


def run_bn254(args, D):
    """BN254 workload: one 16-layer circuit of 2^16 gates (50% mul / 50% add fan-in-2,
    uniform wiring, 64 copies) proved plainly, then 64 independent proofs of widths
    2^12..2^16 (16 layers, 64 copies, own seed each) plain vs batched."""
    from concurrent.futures import ThreadPoolExecutor

    from gkr_gb300 import circuit as gc
    from gkr_gb300.prover import Context, DeviceBuffer, HostBuffer
    if D.rank != 0:
        return
    N, depth_l, width = 64, 16, 16
    ctx = Context(D.local_rank)
    circ = gc.uniform_circuit(4254, depth_l, width, p_mul=0.5)
    dc = ctx.load(circ, "BN254")
    rows = 1 << circ.log_input_size
    plen = dc.proof_size(N)
    hin = HostBuffer(rows * N * 32, np.uint64)
    witness = hin.array.reshape(rows, N, 4)
    witness[:] = gc.random_witness_bn254(4254, circ.log_input_size, N)
    din = DeviceBuffer(ctx, rows * N * 32)
    din.upload(witness)
    pbufs = [HostBuffer(plen) for _ in range(args.depth)]
    bufs = [(pb.array, np.empty((1, N, 4), np.uint64)) for pb in pbufs]
    tiles = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        tiles = ctx.autotune(dc, None, n_copies=N, d_input=din.ptr)
        tiles = {"seconds": time.perf_counter() - t0,
                 "choice": {k: {"threads_per_row": v["threads_per_row"], "ctas": v["ctas"]}
                            for k, v in tiles.items() if v["ms"] > 0}}
        ctx.reset_stats()

    # plain proofs with args.plain_lanes device lanes; per-launch times from a one-lane pass
    one_lane = args.plain_lanes <= 1
    if not one_lane:
        ctx.set_concurrency(lanes=args.plain_lanes)
    ctx.set_timing(one_lane)
    clocks = ClockSampler(D.local_rank)
    clocks.start()
    total_ms, step_ms, lat_ms, s0, s1, _ = pipelined(
        ctx, args.warmup, args.steps, bufs, lambda b, m: ctx.submit(dc, None, b[0], b[1], d_input=din.ptr, marker=m))
    clk = clocks.stop()
    ctx.set_timing(False)
    stats, stat_steps = stats_delta(s0, s1), args.steps
    value = args.steps / (total_ms / 1000.0)
    e2e = None
    if not args.no_e2e:
        h0 = ctx.transfer_stats()
        e2e_warm = max(1, args.warmup)
        e2e_ms, _, e2e_lat, _, _, _ = pipelined(ctx, e2e_warm, args.steps, bufs,
                                               lambda b, m: ctx.submit(dc, witness, b[0], b[1], marker=m))
        h1 = ctx.transfer_stats()
        n_jobs = e2e_warm + args.steps
        e2e = {"value": args.steps / (e2e_ms / 1000.0), "unit": UNIT,
               "h2d_bytes_per_step": (h1[0] - h0[0]) // n_jobs, "d2h_bytes_per_step": (h1[1] - h0[1]) // n_jobs,
               "latency_ms": {"p50": statistics.median(e2e_lat), "p99": float(np.percentile(e2e_lat, 99))}}
    kernel_timing = "per-launch CUDA events on the library's stream inside the timed region"
    if not one_lane:
        ctx.set_concurrency(lanes=1)
        ctx.set_timing(True)
        _, _, _, k0, k1, _ = pipelined(ctx, 1, 2, bufs,
                                       lambda b, m: ctx.submit(dc, None, b[0], b[1], d_input=din.ptr, marker=m))
        ctx.set_timing(False)
        stats, stat_steps = stats_delta(k0, k1), 2
        kernel_timing = (f"per-launch CUDA events in a one-lane pass of 2 proofs after the timed regions (with "
                         f"{args.plain_lanes} lanes another proof's kernels share the GPU)")
    kernels = {k: {"launches_per_step": v["launches"] / stat_steps, "ms_per_step": v["ms"] / stat_steps,
                   "GBps": (v["bytes"] / (v["ms"] / 1000.0) / 1e9) if v["ms"] else None}
               for k, v in stats.items() if v["launches"]}
    peak, peak_kind = peaks()
    name, s = max(stats.items(), key=lambda kv: kv[1]["ms"])
    per_b, per_ms = s["bytes"] / max(s["launches"], 1), s["ms"] / max(s["launches"], 1)
    achieved = per_b / (per_ms / 1000.0) / 1e9 if per_ms > 0 else 0.0
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": None, "peak_source": peak_kind,
                "note": "256-bit Montgomery products make these kernels integer-multiply bound; the HBM fraction "
                        "is reported for comparison"}

    cpu = None
    if not args.no_cpu_baseline:
        from oracle.oracle import OracleBn254
        threads = len(os.sched_getaffinity(0))
        cn = 8
        w8 = gc.random_witness_bn254(7, circ.log_input_size, cn)
        dt = OracleBn254().bench(circ, w8, threads, 1)
        cpu = {"value": threads / dt * cn / N, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{threads} threads x 1 proof of the same circuit at {cn} copies (oracle/gkr_oracle_bn254.c, "
                         f"evaluate + prove), scaled by {cn}/{N} to {N}-copy proofs/s"}

    batched = None
    if not args.no_batched:
        # ---- batched: 64 independent proofs, widths 2^12..2^16
        n_b = 64
        st = gc.Stream(99)
        ks = (12 + st.below(n_b, 5)).tolist()
        with ThreadPoolExecutor(8) as ex:
            circs = list(ex.map(lambda i: gc.uniform_circuit(5000 + i, depth_l, int(ks[i]), p_mul=0.5), range(n_b)))
            wits = list(ex.map(lambda i: gc.random_witness_bn254(5000 + i, int(ks[i]), N), range(n_b)))
        dcs = [ctx.load(c, "BN254") for c in circs]
        pbs = [np.empty(d.proof_size(N), np.uint8) for d in dcs]
        cbs = [np.empty((1, N, 4), np.uint64) for _ in range(n_b)]

        def run_all(lanes):
            ctx.set_concurrency(lanes=lanes, hbm_budget_bytes=int(args.budget_gb * (1 << 30)))
            for i in range(min(lanes, n_b)):
                ctx.wait(ctx.submit(dcs[i], wits[i], pbs[i], cbs[i]))
            lat = []
            t0 = time.perf_counter()
            if lanes == 1:
                for i in range(n_b):
                    t1 = time.perf_counter()
                    ctx.wait(ctx.submit(dcs[i], wits[i], pbs[i], cbs[i]))
                    lat.append((time.perf_counter() - t1) * 1000.0)
            else:
                subs = [(time.perf_counter(), ctx.submit(dcs[i], wits[i], pbs[i], cbs[i])) for i in range(n_b)]
                for t1, j in subs:
                    ctx.wait(j)
                    lat.append((time.perf_counter() - t1) * 1000.0)
            sec = time.perf_counter() - t0
            import hashlib
            return n_b / sec, lat, [hashlib.sha256(p.tobytes()).hexdigest() for p in pbs]

        plain_v, plain_lat, plain_d = run_all(1)
        batch_v, batch_lat, batch_d = run_all(args.lanes)
        batched = {"proofs": n_b, "widths_log2": sorted(set(int(k) for k in ks)), "layers": depth_l,
                   "n_copies": N, "lanes": args.lanes, "proofs_per_s": batch_v,
                   "latency_ms": {"p50": statistics.median(batch_lat), "p99": float(np.percentile(batch_lat, 99))},
                   "plain_proofs_per_s": plain_v,
                   "plain_latency_ms": {"p50": statistics.median(plain_lat),
                                        "p99": float(np.percentile(plain_lat, 99))},
                   "batched_over_plain": batch_v / plain_v, "byte_identical_to_plain": batch_d == plain_d}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u256 (BN254 Montgomery, 8 x u32 limbs)", "data": "synthetic",
            "config": {"workload": f"BN254: {depth_l} layers of 2^{width} gates, 50% mul / 50% add fan-in-2, uniform "
                                   f"wiring, {N} copies, uniform witness in [0, r), SHA-256 transcript, RAW "
                                   "commitment (one plain proof per step)",
                       "n_copies": N, "layers": depth_l, "width_log2": width, "field": "BN254", "repetitions": 1,
                       "grinding_bits": 10,
                       "pipeline": f"{args.depth} proofs in flight, {args.plain_lanes} device lane(s)"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(round(sum(v["launches"] for v in stats.values()) / stat_steps * args.steps)),
            "autotune": tiles, "clocks": clk,
            "latency_ms": {"p50": statistics.median(lat_ms), "p99": float(np.percentile(lat_ms, 99)),
                           "device_end_intervals_ms": step_ms},
            "kernels": kernels, "kernel_timing": kernel_timing, "proof_bytes": plen,
            "batched": batched}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    D = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, D)
        elif args.workload == "mixed":
            run_mixed(args, D)
        elif args.workload == "serve":
            run_serve(args, D)
        elif args.workload == "bn254":
            run_bn254(args, D)
        else:
            run_ours(args, D)
    finally:
        D.close()


if __name__ == "__main__":
    main()
