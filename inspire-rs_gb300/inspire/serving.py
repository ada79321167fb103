"""Load generation and latency accounting for the serving loop.

Open loop: Poisson arrivals at a fixed offered rate, split over several
submitter threads (a superposition of independent Poisson streams is Poisson
at the summed rate); each query is stamped with its scheduled arrival time,
so time spent waiting in a submitter or for a free slot counts as latency.
Closed loop: every submitter keeps submitting as fast as the loop admits,
which measures the saturated end-to-end rate through host buffers.

Queries come from a QueryPool of real seeded queries (rows laid out as the
C ABI takes them); a query's target database is drawn with probability
proportional to its entry count and its shard uniformly, i.e. the queried
index is uniform over all entries.
"""
from __future__ import annotations

import gc
import threading
import time
from collections import deque
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _native as nat
from .pir import now_ns


@dataclass
class Target:
    db: object          # EncodedDatabase
    nshards: int
    weight: float = 1.0


class QueryPool:
    """Q real seeded queries, contiguous: seeds (Q, 2*ell, 32) uint8,
    b_rows (Q, 2*ell, plen) uint64; the entry index each one asks for
    (local index within its shard) in `locals_`.  pinned=True places the
    rows in page-locked memory and submissions borrow them (the GPU reads
    them in place; nothing is copied on the host)."""

    def __init__(self, seeds: np.ndarray, b_rows: np.ndarray, locals_: Sequence[int], pinned: bool = False,
                 client_ids: Optional[Sequence[int]] = None):
        self.locals_ = np.asarray(locals_)
        # registered client id of each query (its packing keys); None: the
        # client_id given to run()
        self.client_ids = None if client_ids is None else np.ascontiguousarray(client_ids, dtype=np.int32)
        self.borrow = pinned
        self._bufs = []
        if pinned:
            from .pir import PinnedBuffer

            sb = PinnedBuffer(seeds.shape, np.uint8)
            bb = PinnedBuffer(b_rows.shape, np.uint64)
            sb.array[:] = seeds
            bb.array[:] = b_rows
            self._bufs = [sb, bb]
            self.seeds, self.b_rows = sb.array, bb.array
        else:
            self.seeds = np.ascontiguousarray(seeds, dtype=np.uint8)
            self.b_rows = np.ascontiguousarray(b_rows, dtype=np.uint64)
        self.q = self.seeds.shape[0]

    def close(self):
        self.seeds = self.b_rows = None
        for b in self._bufs:
            b.close()
        self._bufs = []

    def ranges(self, start: int, m: int):
        """Contiguous pool ranges covering m queries from position start
        (cyclic): list of (lo, hi)."""
        out = []
        pos = start % self.q
        while m > 0:
            take = min(m, self.q - pos)
            out.append((pos, pos + take))
            m -= take
            pos = 0
        return out


def poisson_offsets_ns(rate: float, duration_s: float, rng: np.random.Generator) -> np.ndarray:
    """Arrival offsets (ns, sorted, < duration) of a Poisson process."""
    n_est = int(rate * duration_s * 1.2 + 64)
    gaps = rng.exponential(1.0 / rate, size=n_est)
    t = np.cumsum(gaps)
    while t[-1] < duration_s:
        more = np.cumsum(rng.exponential(1.0 / rate, size=n_est)) + t[-1]
        t = np.concatenate([t, more])
    return (t[t < duration_s] * 1e9).astype(np.int64)


def latency_summary(arrival_ns: np.ndarray, done_ns: np.ndarray) -> dict:
    """p50 / p99 / p99.9 / mean latency (ms) and the achieved rate."""
    a = np.asarray(arrival_ns, dtype=np.int64)
    d = np.asarray(done_ns, dtype=np.int64)
    if a.size == 0:
        return {"n": 0}
    lat = (d - a) / 1e6
    span = (d.max() - a.min()) / 1e9
    return {"n": int(a.size), "achieved_qps": float(a.size / span) if span > 0 else None,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "p999_ms": float(np.percentile(lat, 99.9)), "mean_ms": float(lat.mean()),
            "max_ms": float(lat.max())}


def _choose(targets: List[Target], n: int, rng: np.random.Generator):
    w = np.array([t.weight for t in targets], dtype=np.float64)
    dbi = rng.choice(len(targets), size=n, p=w / w.sum())
    ns = np.array([t.nshards for t in targets], dtype=np.int64)
    shards = np.minimum((rng.random(n) * ns[dbi]).astype(np.int64), ns[dbi] - 1).astype(np.uint32)
    return dbi, shards


class _Lane:
    """One submitter thread and its collector."""

    def __init__(self, server, handles, pool, client_id, arrivals, dbi, shards, max_burst, keep_outputs):
        self.server, self.pool, self.cid = server, pool, client_id
        self.arrivals, self.dbi, self.shards = arrivals, dbi, shards
        self.hdl = handles[dbi]       # per-query database handle values
        self.max_burst = max_burst
        self.keep = keep_outputs
        self.queue = deque()          # (tickets, arrival_ns, pool_idx, db_idx, shard) chunks for the collector
        self.cv = threading.Condition()
        self.submitted_all = False
        self.done_arrival, self.done_at, self.done_submit = [], [], []
        self.samples = []             # (db_idx, shard, pool_idx, out) of kept outputs
        self.error: Optional[BaseException] = None
        self.pool_pos = 0
        self.cids = np.full(max(max_burst, pool.q), client_id, np.int32)

    def _submit(self, i: int, j: int):
        """Submit arrivals i..j-1 (any databases) in contiguous pool ranges,
        retrying on backpressure."""
        k = i
        for lo, hi in self.pool.ranges(self.pool_pos, j - i):
            off = 0
            m = hi - lo
            while off < m:
                a, b = k + off, k + m
                plo = lo + off
                t_sub = now_ns()
                cids = self.cids[:b - a] if self.pool.client_ids is None else self.pool.client_ids[plo:hi]
                t, rc = self.server.submit(self.hdl[a:b], self.shards[a:b], self.pool.seeds[plo:hi],
                                           self.pool.b_rows[plo:hi], cids,
                                           self.arrivals[a:b] if self.arrivals is not None else None,
                                           borrow=self.pool.borrow)
                if len(t):
                    arr = self.arrivals[a:a + len(t)] if self.arrivals is not None else \
                        np.full(len(t), t_sub, np.int64)
                    sub = np.full(len(t), t_sub, np.int64)
                    with self.cv:
                        self.queue.append((t, arr, sub, np.arange(plo, plo + len(t)), self.dbi[a:a + len(t)],
                                           self.shards[a:a + len(t)]))
                        self.cv.notify()
                off += len(t)
                if rc == nat.ERR_BUSY:
                    time.sleep(50e-6)
                elif rc != nat.OK:
                    raise RuntimeError(f"submit failed with status {rc}: {nat.last_error()}")
            k += m
        self.pool_pos += j - i

    def submitter(self):
        try:
            n = len(self.dbi)
            i = 0
            while i < n:
                if self.arrivals is not None:
                    now = now_ns()
                    if self.arrivals[i] > now:
                        time.sleep(min(1e-3, (self.arrivals[i] - now) / 1e9))
                        continue
                    j = int(np.searchsorted(self.arrivals, now, side="right"))
                else:
                    j = n
                j = min(j, i + self.max_burst)
                self._submit(i, j)
                i = j
        except BaseException as e:  # reported by run()
            self.error = e
        finally:
            with self.cv:
                self.submitted_all = True
                self.cv.notify()

    def collector(self):
        try:
            while True:
                with self.cv:
                    while not self.queue and not self.submitted_all:
                        self.cv.wait(0.01)
                    if not self.queue and self.submitted_all:
                        return
                    t, arr, sub, pidx, d, sh = self.queue.popleft()
                got = 0
                out = np.zeros((len(t), 2, self.pool.b_rows.shape[-1]), np.uint64) if self.keep else None
                while got < len(t):
                    o = None if out is None else out[got:]
                    done = self.server.poll_batch(t[got:], o, timeout_us=2000)
                    self.done_arrival.append(arr[got:got + len(done)])
                    self.done_submit.append(sub[got:got + len(done)])
                    self.done_at.append(done)
                    got += len(done)
                if self.keep:
                    for k in range(len(t)):
                        self.samples.append((int(d[k]), int(sh[k]), int(pidx[k]), out[k]))
                    self.keep = False  # one chunk per lane is enough to check
        except BaseException as e:
            self.error = e


def run(server, targets: List[Target], pool: QueryPool, client_id: int, *, rate: Optional[float],
        duration_s: float = 2.0, n_queries: int = 0, n_threads: int = 4, max_burst: int = 256, seed: int = 0,
        keep_outputs: bool = False, closed_chunk: int = 128, settle_frac: float = 0.1) -> dict:
    """Open loop at `rate` q/s for duration_s, or (rate None) closed loop
    over n_queries submitted closed_chunk at a time.  Returns
    latency_summary() plus the offered rate and, if keep_outputs, a few
    (db_idx, shard, pool_idx, response) samples.  Open-loop statistics skip
    the queries that arrive in the first settle_frac of the run (threads
    starting, first launches)."""
    rng = np.random.default_rng(seed)
    handles = np.array([server.handle_of(t.db) for t in targets], dtype=np.uint64)
    plans = []
    for k in range(n_threads):
        if rate is not None:
            offs = poisson_offsets_ns(rate / n_threads, duration_s, rng)
            n = len(offs)
        else:
            offs = None
            n = n_queries // n_threads
        plans.append((offs,) + _choose(targets, n, rng))
    # arrival times are fixed only once every lane's schedule is built, with
    # 20 ms for the threads to start
    t0 = now_ns() + 20_000_000
    lanes = [_Lane(server, handles, pool, client_id, None if offs is None else t0 + offs, dbi, shards,
                   max_burst if rate is not None else closed_chunk, keep_outputs) for offs, dbi, shards in plans]
    # the cyclic garbage collector stops every load-generator thread while it
    # runs (tens of ms in a large process); it stays off during the run
    gc_was_enabled = gc.isenabled()
    gc.disable()
    try:
        wall0 = time.perf_counter()
        ths = []
        for ln in lanes:
            ths.append(threading.Thread(target=ln.submitter))
            ths.append(threading.Thread(target=ln.collector))
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        wall = time.perf_counter() - wall0
    finally:
        if gc_was_enabled:
            gc.enable()
    for ln in lanes:
        if ln.error is not None:
            raise ln.error
    arr = np.concatenate([np.concatenate(ln.done_arrival) for ln in lanes if ln.done_arrival])
    done = np.concatenate([np.concatenate(ln.done_at) for ln in lanes if ln.done_at])
    sub = np.concatenate([np.concatenate(ln.done_submit) for ln in lanes if ln.done_submit])
    n_all = int(arr.size)
    if rate is not None and settle_frac > 0:
        keep = arr >= t0 + int(settle_frac * duration_s * 1e9)
        arr, done, sub = arr[keep], done[keep], sub[keep]
    res = latency_summary(arr, done)
    if rate is not None and sub.size:
        # from the submit call instead of the scheduled arrival: the server's
        # own latency, without the load generator's lag in submitting
        srv = latency_summary(sub, done)
        res["from_submit_p50_ms"], res["from_submit_p99_ms"] = srv["p50_ms"], srv["p99_ms"]
    res["n_total"] = n_all
    res["offered_qps"] = rate
    res["wall_s"] = wall
    if keep_outputs:
        res["samples"] = [s for ln in lanes for s in ln.samples]
    return res


def autotune(make_server, targets: List[Target], pool: QueryPool, client_id: int, *,
             batches=(128, 152, 256), inflight=(4, 8), waits_us=(25, 100), n_queries: int = 1 << 15,
             n_threads: int = 4, tie: float = 0.01) -> dict:
    """Pick the serving configuration (max_batch, max_inflight,
    batch_wait_us) by saturated closed-loop rate: among the candidates within
    `tie` (relative) of the highest rate, the one with the most batches in
    flight, then the smallest batches (under partial load a partial batch
    launches at once while a stream is free, so more streams and smaller
    batches mean less waiting).  make_server(max_batch=, max_inflight=,
    batch_wait_us=) builds a server; each candidate gets a warm-up run, then
    a timed run of n_queries.  Returns {"best": config, "table": [config +
    rate, ...]}."""
    table = []
    for mb in batches:
        for mi in inflight:
            for w in waits_us:
                srv = make_server(max_batch=mb, max_inflight=mi, batch_wait_us=w)
                try:
                    run(srv, targets, pool, client_id, rate=None, n_queries=n_queries // 4, n_threads=n_threads)
                    r = run(srv, targets, pool, client_id, rate=None, n_queries=n_queries, n_threads=n_threads,
                            closed_chunk=min(pool.q, 256))
                finally:
                    srv.close()
                table.append({"max_batch": mb, "max_inflight": mi, "batch_wait_us": w,
                              "qps": r["achieved_qps"], "p50_ms": r["p50_ms"]})
    return {"best": pick_config(table, tie), "table": table}


def pick_config(table: List[dict], tie: float = 0.01) -> dict:
    """autotune's choice from its table (rows with max_batch, max_inflight,
    batch_wait_us and qps)."""
    top = max(t["qps"] for t in table)
    near = [t for t in table if t["qps"] >= (1.0 - tie) * top]
    best = min(near, key=lambda t: (-t["max_inflight"], t["max_batch"], t["batch_wait_us"]))
    return {k: best[k] for k in ("max_batch", "max_inflight", "batch_wait_us")}

def run_native(server, targets: List[Target], pool: QueryPool, client_id: int, *, rate: float,
               duration_s: float = 2.0, seed: int = 0, keep_outputs: bool = False, settle_frac: float = 0.1,
               max_burst: int = 256) -> dict:
    """Open loop at `rate` q/s for duration_s, driven by the library's native
    submitter and collector threads (Server.drive): Poisson arrivals, query
    k on pool entry k mod Q, database and shard drawn as in run().  Returns
    latency_summary() from the scheduled arrival, the same from the
    submission call (from_submit_*), the offered rate and, if keep_outputs,
    a few (db_idx, shard, pool_idx, response) samples."""
    rng = np.random.default_rng(seed)
    handles = np.array([server.handle_of(t.db) for t in targets], dtype=np.uint64)
    offs = poisson_offsets_ns(rate, duration_s, rng)
    n = len(offs)
    dbi, shards = _choose(targets, n, rng)
    pidx = np.arange(n) % pool.q
    cids = pool.client_ids[pidx] if pool.client_ids is not None else np.full(n, client_id, np.int32)
    t0 = now_ns() + 20_000_000
    arrivals = t0 + offs
    n_keep = min(16, n) if keep_outputs else 0
    gc_was_enabled = gc.isenabled()
    gc.disable()
    try:
        sub, done, kept = server.drive(handles[dbi], shards, cids, pool.seeds, pool.b_rows, arrivals,
                                       borrow=pool.borrow, max_burst=max_burst, n_keep=n_keep)
    finally:
        if gc_was_enabled:
            gc.enable()
    keep = arrivals >= t0 + int(settle_frac * duration_s * 1e9)
    out = latency_summary(arrivals[keep], done[keep])
    fs = latency_summary(sub[keep], done[keep])
    out.update({"from_submit_p50_ms": fs.get("p50_ms"), "from_submit_p99_ms": fs.get("p99_ms"),
                "n_total": int(n), "offered_qps": rate, "driver": "native (Server.drive)"})
    if keep_outputs:
        out["samples"] = [(int(dbi[k]), int(shards[k]), int(pidx[k]), kept[k]) for k in range(n_keep)]
    return out
