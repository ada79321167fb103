"""Load generator for the HTTP front end: client processes (spawned, so they
do not share the server's interpreter) posting prepared JSON query bodies
over keep-alive connections, closed loop (each connection sends its next
query when the previous reply has arrived) or open loop (Poisson arrivals
at a given total rate; latency counted from the scheduled arrival).

Bodies are SeededClientQuery JSON as the crate's client sends them
(src/bin/client.rs posts serde_json of the query, keys included)."""
from __future__ import annotations

import http.client
import multiprocessing as mp
import os
import tempfile
import threading
import time
from typing import Sequence

import numpy as np

Q_MODULI = (268369921, 249561089)


def _poly_json(coeffs, n: int) -> str:
    q0, q1 = Q_MODULI
    inv = pow(q0, q1 - 2, q1)
    return ('{"coeffs":[' + ",".join(map(str, np.asarray(coeffs).tolist())) + '],"moduli":[%d,%d],"q":%d,"dim":%d,'
            '"crt_q0_inv_mod_q1":%d,"is_ntt":false}' % (q0, q1, q0 * q1, n, inv))


def seeded_query_json(shard_id: int, seeds: np.ndarray, b_rows: np.ndarray, y_body: np.ndarray,
                      n: int = 2048, mode: str = "inspiring") -> bytes:
    """serde_json of SeededClientQuery (pir/query.rs:138-150) with
    inspiring_packing_keys {y_body}, compact form."""
    rows = ",".join('{"seed":[' + ",".join(map(str, seeds[i].tolist())) + '],"b":' + _poly_json(b_rows[i], n) + "}"
                    for i in range(seeds.shape[0]))
    q0, q1 = Q_MODULI
    keys = '{"y_body":[' + ",".join(_poly_json(p, n) for p in y_body) + '],"full_key":false,"num_to_pack":16}'
    return ('{"shard_id":%d,"rgsw_ciphertext":{"rows":[%s],"gadget":{"base":1048576,"len":3,"q":%d}},'
            '"packing_mode":"%s","inspiring_packing_keys":%s}' % (shard_id, rows, q0 * q1, mode, keys)).encode()


def _worker(host, port, path, bodies_file, offsets, threads, duration_s, warmup_s, rate, seed, out_q):
    with open(bodies_file, "rb") as f:
        blob = f.read()
    bodies = [blob[offsets[i]:offsets[i + 1]] for i in range(len(offsets) - 1)]
    t_start = time.monotonic() + 0.2
    t_end = t_start + warmup_s + duration_s
    results = [[] for _ in range(threads)]
    errors = [0] * threads

    def run(t):
        conn = http.client.HTTPConnection(host, port, timeout=60)
        rng = np.random.default_rng(seed * 1000 + t)
        k = (seed * 7919 + t * 104729) % len(bodies)
        nxt = t_start + (rng.exponential(threads / rate) if rate else 0.0)
        while True:
            if rate:  # open loop: send at the scheduled arrival (or at once when late)
                now = time.monotonic()
                if nxt >= t_end:
                    break
                if nxt > now:
                    time.sleep(nxt - now)
                sched = nxt
                nxt += rng.exponential(threads / rate)
            else:
                sched = time.monotonic()
                if sched >= t_end:
                    break
            body = bodies[k]
            k = (k + 1) % len(bodies)
            conn.request("POST", path, body=body, headers={"Content-Type": "application/json"})
            r = conn.getresponse()
            r.read()
            done = time.monotonic()
            if r.status != 200:
                errors[t] += 1
            elif sched >= t_start + warmup_s:
                results[t].append((sched, done - sched))
        conn.close()

    ths = [threading.Thread(target=run, args=(t,)) for t in range(threads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    lat = [x for r in results for x in r]
    out_q.put((lat, sum(errors)))


def run_load(url: str, bodies: Sequence[bytes], connections: int, duration_s: float = 2.0, warmup_s: float = 0.5,
             rate: float = 0.0, processes: int = 0, path: str = "/query_seeded") -> dict:
    """Drive `connections` keep-alive connections (spread over `processes`
    spawned client processes) for duration_s after warmup_s.  rate = 0:
    closed loop; rate > 0: open loop with Poisson arrivals at `rate`
    requests/s in total.  Returns achieved requests/s, p50/p99/p999 latency
    (ms) and the count of non-200 replies."""
    host, port = url.split("//")[1].split(":")
    procs = processes or min(connections, max(1, (os.cpu_count() or 2) // 2))
    procs = max(1, min(procs, connections))
    per = [connections // procs + (1 if i < connections % procs else 0) for i in range(procs)]
    fd, bodies_file = tempfile.mkstemp(prefix="inspire_http_bodies_")
    offsets = [0]
    with os.fdopen(fd, "wb") as f:
        for b in bodies:
            f.write(b)
            offsets.append(offsets[-1] + len(b))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(host, int(port), path, bodies_file, offsets, per[i], duration_s, warmup_s,
                                             rate * per[i] / connections if rate else 0.0, i, q))
          for i in range(procs)]
    try:
        for p in ps:
            p.start()
        lat, errors = [], 0
        for _ in ps:
            l_, e = q.get(timeout=duration_s + warmup_s + 120)
            lat.extend(l_)
            errors += e
        for p in ps:
            p.join()
    finally:
        os.unlink(bodies_file)
    ms = np.array([d for _, d in lat]) * 1e3 if lat else np.zeros(1)
    return {"connections": connections, "client_processes": procs, "offered_rps": rate or None,
            "achieved_rps": len(lat) / duration_s, "requests": len(lat), "errors": errors,
            "p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99)),
            "p999_ms": float(np.percentile(ms, 99.9)), "mean_ms": float(ms.mean())}


__all__ = ["seeded_query_json", "run_load"]
