"""Serving: a request loop over one context with continuous batching.

Requests (a loaded circuit and a witness) arrive from any thread.  Device memory is
admitted in two steps, both by footprint:
* a request is admitted when its witness fits the device arena (and fewer than
  `max_admitted` requests are in flight): the witness is uploaded once (gkrgpu_upload, on
  the context's transfer stream, while other proofs run), stays resident until the proof is
  done, and the proof is queued with gkrgpu_prove_submit_resident, so its host stage (the
  SHA-256 of the RAW commitment, from the caller's host copy) starts at once;
* its device stage starts when a lane is free and the proof's workspace
  (gkrgpu_workspace_bytes: every layer's values and the sumcheck tables) fits the HBM budget
  next to the running ones (gkrgpu_set_concurrency); the device stage computes from the
  resident witness, so nothing is copied per proof besides the round rows the transcript
  needs.
Up to `lanes` proofs run their device stages at once and whatever is pending is taken into
the lanes as earlier proofs finish, whatever its size.  Requests beyond `max_queue` waiting
for admission are rejected (admission control), and every result carries its latency.
Proof buffers come from a pool the server keeps by size class (powers of two from 1 MiB): a
caller done with a result hands its buffer back with Result.release(), so a steady stream of
requests, of any mix of sizes, writes its proofs into memory that is already mapped (a fresh
multi-megabyte buffer per request pays first-touch page faults, which stall for long when the
host is reclaiming or compacting memory).

The reference has no serving loop (benchmarks/bench_keccak.cpp:32-42 proves in a closed
loop, one proof per thread).
"""
import threading
import time
from collections import deque
from concurrent.futures import Future

import numpy as np

from .prover import DeviceBuffer, _table

ALIGN = 256


class Rejected(RuntimeError):
    """The admission queue was full when the request arrived."""


class Arena:
    """First-fit sub-allocator of one device buffer (offsets aligned to 256 bytes, free
    neighbours merged).  Not thread-safe: the server calls it under its lock."""

    def __init__(self, size: int):
        self.size = size
        self.free = [(0, size)]  # sorted (offset, length)
        self.used = {}

    def alloc(self, nbytes: int):
        n = -(-max(nbytes, 1) // ALIGN) * ALIGN
        for i, (off, ln) in enumerate(self.free):
            if ln >= n:
                if ln == n:
                    del self.free[i]
                else:
                    self.free[i] = (off + n, ln - n)
                self.used[off] = n
                return off
        return None

    def release(self, off: int):
        n = self.used.pop(off)
        self.free.append((off, n))
        self.free.sort()
        merged = []
        for o, ln in self.free:
            if merged and merged[-1][0] + merged[-1][1] == o:
                merged[-1] = (merged[-1][0], merged[-1][1] + ln)
            else:
                merged.append((o, ln))
        self.free = merged

    def in_use(self) -> int:
        return sum(self.used.values())


class BufferPool:
    """Host buffers for proofs, kept by size class (the next power of two of at least 1 MiB)
    up to `cap_bytes` in all.  Not thread-safe: the server calls it under its lock."""

    MIN_CLASS = 1 << 20

    def __init__(self, cap_bytes: int):
        self.cap = cap_bytes
        self.free = {}  # class size -> [buffers]
        self.pooled = 0

    @classmethod
    def size_class(cls, nbytes: int) -> int:
        c = cls.MIN_CLASS
        while c < nbytes:
            c <<= 1
        return c

    def take(self, nbytes: int):
        """A pooled buffer of nbytes' class, or None."""
        c = self.size_class(nbytes)
        bufs = self.free.get(c)
        if not bufs:
            return None
        self.pooled -= c
        return bufs.pop()

    def give(self, buf) -> bool:
        """Keeps `buf` (of a class size) unless the pool is full; returns whether it was kept."""
        if buf.size != self.size_class(buf.size) or self.pooled + buf.size > self.cap:
            return False
        self.free.setdefault(buf.size, []).append(buf)
        self.pooled += buf.size
        return True


class Result:
    """A finished request: claimed values (R, N), the proof bytes (uint8 array) and times."""

    def __init__(self, claimed_v, proof, latency_ms, admit_wait_ms, server=None, buf=None):
        self.claimed_v = claimed_v
        self.proof = proof
        self.latency_ms = latency_ms
        self.admit_wait_ms = admit_wait_ms
        self._server, self._buf = server, buf

    def release(self):
        """Hands the proof buffer back to the server for later requests; `proof` must not be
        used afterwards."""
        if self._server is not None and self._buf is not None:
            self._server._give_back(self._buf)
        self.proof, self._server, self._buf = None, None, None


class _Req:
    def __init__(self, dc, witness, grinding_bits):
        self.dc = dc
        self.witness = _table(dc.field, witness)
        self.grinding_bits = grinding_bits
        self.n = self.witness.shape[1]
        self.wbytes = self.witness.nbytes
        self.t_arr = time.perf_counter()
        self.t_adm = None
        self.future = Future()
        self.off = None
        self.job = None
        self.proof = None
        self.claims = None


class ProofServer:
    """The request loop.  `arena_bytes` of device memory hold the resident witnesses of the
    admitted requests; `budget_bytes` bounds the workspaces of the proofs whose device stages
    run (a proof larger than the whole budget runs alone); `max_admitted` (None: no bound)
    caps the requests in flight."""

    def __init__(self, ctx, lanes=16, budget_bytes=150 << 30, arena_bytes=16 << 30, max_queue=1 << 20,
                 max_admitted=None, pool_bytes=16 << 30):
        self.ctx = ctx
        self.lanes = lanes
        self.budget = budget_bytes
        self.max_queue = max_queue
        self.max_admitted = max_admitted
        ctx.set_concurrency(lanes=lanes, hbm_budget_bytes=budget_bytes)
        self.buf = DeviceBuffer(ctx, arena_bytes)
        self.arena = Arena(arena_bytes)
        self.cv = threading.Condition()
        self.pending = deque()  # arrived, not admitted
        self.running = deque()  # admitted, waiting for a waiter thread
        self.in_flight = 0
        self.peak = 0
        self.admitted = 0
        self.rejected = 0
        self.completed = 0
        self.stopping = False
        self.pool = BufferPool(pool_bytes)  # proof buffers handed back
        self.threads = [threading.Thread(target=self._admit_loop, daemon=True)]
        self.threads += [threading.Thread(target=self._wait_loop, daemon=True) for _ in range(lanes)]
        for t in self.threads:
            t.start()

    # ---------------------------------------------------------------- API
    def submit(self, dc, witness, grinding_bits=10) -> Future:
        """Queues one proof; the future's result is a Result, or Rejected when the admission
        queue is full."""
        r = _Req(dc, witness, grinding_bits)
        if r.wbytes > self.arena.size:
            r.future.set_exception(ValueError(f"witness of {r.wbytes} bytes exceeds the arena"))
            return r.future
        with self.cv:
            if self.stopping:
                raise RuntimeError("server is closed")
            if len(self.pending) >= self.max_queue:
                self.rejected += 1
                r.future.set_exception(Rejected("admission queue full"))
                return r.future
            self.pending.append(r)
            self.cv.notify_all()
        return r.future

    def drain(self):
        """Waits until every accepted request has finished."""
        with self.cv:
            self.cv.wait_for(lambda: not self.pending and not self.running and self.in_flight == 0)

    def close(self):
        self.drain()
        with self.cv:
            self.stopping = True
            self.cv.notify_all()
        for t in self.threads:
            t.join()
        self.buf.free()

    def stats(self):
        """Request counts, the peak of resident witness bytes, and the library's workspace peak."""
        mem = self.ctx.memory_stats()
        with self.cv:
            return {"admitted": self.admitted, "rejected": self.rejected, "completed": self.completed,
                    "witness_peak_bytes": self.peak, "arena_bytes": self.arena.size,
                    "workspace_peak_bytes": mem["peak"], "budget_bytes": self.budget}

    # ---------------------------------------------------------------- proof buffers
    def _take(self, size):
        with self.cv:
            buf = self.pool.take(size)
        return buf if buf is not None else np.empty(BufferPool.size_class(size), np.uint8)

    def _give_back(self, buf):
        with self.cv:
            self.pool.give(buf)

    # ---------------------------------------------------------------- threads
    def _fits(self):
        return self.max_admitted is None or self.in_flight < self.max_admitted

    def _admit_loop(self):
        while True:
            with self.cv:
                while True:
                    if self.stopping and not self.pending:
                        return
                    if self.pending and self._fits():
                        r = self.pending[0]
                        off = self.arena.alloc(r.wbytes)
                        if off is not None:
                            self.pending.popleft()
                            r.off = off
                            self.in_flight += 1
                            self.peak = max(self.peak, self.arena.in_use())
                            break
                    self.cv.wait()
            try:
                r.t_adm = time.perf_counter()
                d_in = self.buf.ptr + r.off
                w = r.witness
                self.ctx.upload(d_in, w)
                r.proof = self._take(r.dc.proof_size(r.n, r.grinding_bits))
                r.claims = np.empty((r.dc.num_repetitions(r.grinding_bits),) + w.shape[1:], w.dtype)
                r.job = self.ctx.submit_resident(r.dc, w, d_in, r.proof, r.claims, grinding_bits=r.grinding_bits)
            except Exception as e:  # noqa: BLE001 - the request fails, the loop goes on
                self._finish(r, error=e)
                continue
            with self.cv:
                self.admitted += 1
                self.running.append(r)
                self.cv.notify_all()

    def _wait_loop(self):
        while True:
            with self.cv:
                self.cv.wait_for(lambda: self.running or (self.stopping and not self.pending))
                if not self.running:
                    return
                r = self.running.popleft()
            try:
                n = self.ctx.wait(r.job)
                self._finish(r, length=n)
            except Exception as e:  # noqa: BLE001
                self._finish(r, error=e)

    def _finish(self, r, length=None, error=None):
        t = time.perf_counter()
        with self.cv:
            if r.off is not None:
                self.arena.release(r.off)
                self.in_flight -= 1
            self.completed += 1
            self.cv.notify_all()
        if error is not None:
            r.future.set_exception(error)
        else:
            r.future.set_result(Result(r.claims, r.proof[:length], (t - r.t_arr) * 1000.0,
                                       ((r.t_adm or t) - r.t_arr) * 1000.0, self, r.proof))
