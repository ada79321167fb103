"""Host logic of the serving load generator (no GPU): Poisson schedules,
pool ranges, latency summaries, and a full open/closed-loop run against a
fake server with backpressure that checks every query is answered once,
for its own database, shard and pool slot."""
import sys
import threading

import numpy as np
import pytest


@pytest.fixture(scope="module")
def serving():
    sys.path.insert(0, "inspire-rs_gb300")
    from inspire import serving

    return serving


class FakeServer:
    """Admits up to `capacity` outstanding queries (ERR_BUSY beyond), answers
    each with (db tag, shard, first b-row word) after a fixed delay."""

    def __init__(self, capacity=64, delay_ns=200_000):
        from inspire import _native as nat
        from inspire.pir import now_ns

        self.nat, self.now_ns = nat, now_ns
        self.capacity, self.delay = capacity, delay_ns
        self.lock = threading.Lock()
        self.live = {}
        self.next = 1
        self.answers = []

    def handle_of(self, db):
        return {"A": 7, "B": 9}[db]

    def submit(self, dbs, shard_ids, seeds, b_rows, client_ids, arrival_ns=None, borrow=False):
        assert len(dbs) == len(shard_ids) == len(seeds) == len(b_rows) == len(client_ids)
        with self.lock:
            room = self.capacity - len(self.live)
            k = min(room, len(shard_ids))
            t = np.arange(self.next, self.next + k, dtype=np.uint64)
            self.next += k
            now = self.now_ns()
            for j in range(k):
                db = {7: "A", 9: "B"}[int(dbs[j])]
                self.live[int(t[j])] = (now + self.delay, db, int(shard_ids[j]), int(b_rows[j][3][0]))
        return t, (self.nat.OK if k == len(shard_ids) else self.nat.ERR_BUSY)

    def poll_batch(self, tickets, out=None, timeout_us=-1):
        done = []
        for tk in tickets:
            with self.lock:
                t_ready, db, shard, word = self.live[int(tk)]
            while self.now_ns() < t_ready:
                pass
            with self.lock:
                del self.live[int(tk)]
                self.answers.append((db, shard, word))
            if out is not None:
                out[len(done)][0][0] = word
            done.append(t_ready)
        return np.array(done, dtype=np.int64)


def make_pool(serving, q=8):
    seeds = np.zeros((q, 6, 32), np.uint8)
    brows = np.zeros((q, 6, 16), np.uint64)
    brows[:, 3, 0] = np.arange(q) + 1000
    return serving.QueryPool(seeds, brows, np.arange(q))


def test_poisson_schedule_rate(serving):
    rng = np.random.default_rng(0)
    offs = serving.poisson_offsets_ns(20000.0, 2.0, rng)
    assert np.all(np.diff(offs) >= 0) and offs[-1] < 2e9
    assert abs(len(offs) - 40000) < 4 * np.sqrt(40000)
    gaps = np.diff(offs) / 1e9
    assert abs(gaps.mean() - 1 / 20000.0) < 0.05 / 20000.0


def test_pool_ranges_cover_cyclically(serving):
    pool = make_pool(serving, 8)
    assert pool.ranges(6, 5) == [(6, 8), (0, 3)]
    assert pool.ranges(16, 3) == [(0, 3)]
    assert sum(hi - lo for lo, hi in pool.ranges(3, 21)) == 21


def test_latency_summary(serving):
    a = np.arange(1000, dtype=np.int64) * 1_000_000
    d = a + np.where(np.arange(1000) < 990, 1_000_000, 10_000_000)
    s = serving.latency_summary(a, d)
    assert s["n"] == 1000 and s["p50_ms"] == pytest.approx(1.0)
    assert s["p99_ms"] > 1.0 and s["max_ms"] == pytest.approx(10.0)


@pytest.mark.parametrize("rate", [None, 3000.0])
def test_run_against_fake_server(serving, rate):
    pool = make_pool(serving)
    srv = FakeServer(capacity=16)
    targets = [serving.Target("A", 3, 1.0), serving.Target("B", 50, 3.0)]
    res = serving.run(srv, targets, pool, 0, rate=rate, duration_s=0.5, n_queries=400, n_threads=2,
                      seed=1, keep_outputs=True)
    assert res["n_total"] == len(srv.answers) and not srv.live
    if rate is None:
        assert res["n"] == 400
    else:
        assert abs(res["n_total"] - 1500) < 5 * np.sqrt(1500)
        assert abs(res["n"] - 0.9 * 1500) < 5 * np.sqrt(1500)  # the first 10% of arrivals are not counted
        assert res["p50_ms"] >= 0.2
        # submit happens at or after the scheduled arrival
        assert 0 < res["from_submit_p50_ms"] <= res["p50_ms"] + 1e-9
    for db, shard, word in srv.answers:
        assert shard < (3 if db == "A" else 50)
        assert 1000 <= word < 1008
    dbs = [a[0] for a in srv.answers]
    assert 0.6 < dbs.count("B") / len(dbs) < 0.9  # weights 1 : 3
    for db_idx, shard, pidx, out in res["samples"]:
        assert out[0][0] == 1000 + pidx
        assert shard < (3, 50)[db_idx]


def test_device_memory_ledger_host(tmp_path):
    """The context's device-memory accounting (csrc/ledger.h) on the host:
    reservations up to the budget, refusal beyond it with nothing reserved,
    release, and concurrent reservations that never pass the budget; a C++
    driver built with g++."""
    import os
    import shutil
    import subprocess

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    here = os.path.dirname(os.path.abspath(__file__))
    csrc = os.path.join(os.path.dirname(here), "inspire-rs_gb300", "csrc")
    exe = str(tmp_path / "ledger_check")
    subprocess.run([gxx, "-std=c++17", "-O2", "-pthread", "-I", csrc, os.path.join(here, "native", "ledger_check.cpp"),
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout


def test_dispatch_policy_on_host(tmp_path):
    """The serving loop's dispatch decisions (csrc/serve_policy.h) on the
    host, for a 152-SM device: a partial batch goes at once while SMs are
    idle and otherwise after its wait; a batch takes the two-CTA cluster
    kernel only up to pair_max queries and when its SMs are idle, with a
    quarter of the SMs of slack while at most half are busy; a C++ driver
    built with g++."""
    import os
    import shutil
    import subprocess

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    here = os.path.dirname(os.path.abspath(__file__))
    csrc = os.path.join(os.path.dirname(here), "inspire-rs_gb300", "csrc")
    exe = str(tmp_path / "serve_policy_check")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", csrc, os.path.join(here, "native", "serve_policy_check.cpp"),
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout


def test_autotune_pick_prefers_more_streams_on_near_ties(serving):
    """Within the tie band the choice has the most batches in flight, then
    the smallest batches; outside it the rate decides."""
    pick = serving.pick_config
    row = lambda mb, mi, q: {"max_batch": mb, "max_inflight": mi, "batch_wait_us": 100, "qps": q}
    table = [row(128, 4, 917_630.0), row(128, 8, 917_649.0), row(152, 4, 917_040.0), row(152, 8, 915_908.0),
             row(256, 4, 918_109.0), row(256, 8, 918_089.0)]
    assert pick(table) == {"max_batch": 128, "max_inflight": 8, "batch_wait_us": 100}
    table.append(row(256, 4, 990_000.0))  # clearly faster: the rate decides
    assert pick(table) == {"max_batch": 256, "max_inflight": 4, "batch_wait_us": 100}
    assert pick([row(128, 4, 1.0)], tie=0.0) == {"max_batch": 128, "max_inflight": 4, "batch_wait_us": 100}
