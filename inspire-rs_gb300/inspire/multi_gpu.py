"""One database served by several GPUs of a node, partitioned by shard.

A query reads exactly one shard (respond.rs:301-305; ShardConfig::
index_to_shard, params.rs:553-558), so each GPU holds a contiguous range of
shards (ShardRouter) with its own device context, resident partition and
serving loop, and a batch of queries is split by owning GPU on the host.
Nothing crosses between GPUs on the data path: each response is produced
entirely by the GPU that holds its shard, and equals the one-GPU response.

Client packing keys are registered on every partition (any partition may
answer any client); MultiGpuServer maps its client ids to each partition's.
Several partitions may share one device (each with its own context), which
is how this is tested on a single GPU.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from .params import InspireParams
from .pir import ClientPackingKeys, EncodedDatabase, Server, ServerCrs
from .routing import ShardRouter

TICKET_DTYPE = np.dtype([("part", np.uint32), ("ticket", np.uint64)])


class ShardedDatabase:
    """The raw database's shards split into len(devices) contiguous ranges,
    partition p resident on devices[p] (one ServerCrs context each)."""

    def __init__(self, params: InspireParams, inspiring_w_seed: bytes, inspiring_num_columns: int, database,
                 entry_size: int, devices: Sequence[int], mode: str = "crt_fixed"):
        raw = np.frombuffer(database, dtype=np.uint8) if isinstance(database, (bytes, bytearray)) else \
            np.ascontiguousarray(database, dtype=np.uint8).reshape(-1)
        n = params.ring_dim
        self.params = params
        self.entry_size = int(entry_size)
        self.total_entries = raw.size // self.entry_size
        self.num_shards = -(-self.total_entries // n)
        self.router = ShardRouter(n, self.num_shards, len(devices))
        spr = self.router.shards_per_rank()
        self.crs: list[ServerCrs] = []
        self.dbs: list[EncodedDatabase] = []
        for p, dev in enumerate(devices):
            lo, hi = p * spr, min((p + 1) * spr, self.num_shards)
            crs = ServerCrs(params, inspiring_w_seed, inspiring_num_columns, mode=mode, device=dev)
            part = raw[lo * n * self.entry_size:min(hi * n, self.total_entries) * self.entry_size]
            self.crs.append(crs)
            self.dbs.append(EncodedDatabase(crs, part, self.entry_size))

    @property
    def partitions(self) -> int:
        return len(self.dbs)

    def close(self):
        for d in self.dbs:
            d.close()
        for c in self.crs:
            c.close()


class MultiGpuServer:
    """Serving loops over a ShardedDatabase, one per partition: submit()
    splits queries by owning partition (global shard ids), poll_batch()
    collects them in the caller's order."""

    def __init__(self, sdb: ShardedDatabase, servers: Optional[list] = None, **server_kw):
        self.sdb = sdb
        self.router = sdb.router
        self.servers = servers if servers is not None else [Server(c, **server_kw) for c in sdb.crs]
        self._clients: list[list[int]] = []  # global client id -> per-partition ids

    def register_client(self, keys: ClientPackingKeys) -> int:
        ids = [c.register_client(keys) for c in self.sdb.crs]
        self._clients.append(ids)
        return len(self._clients) - 1

    def release_client(self, client_id: int) -> None:
        for c, i in zip(self.sdb.crs, self._clients[client_id]):
            c.release_client(i)

    def submit(self, shard_ids, seeds: np.ndarray, b_rows: np.ndarray, client_ids) -> np.ndarray:
        """Submit n queries with global shard ids; returns n tickets
        (TICKET_DTYPE: owning partition, that partition's ticket).  Raises
        KeyError("Shard {id} not found") for an unknown shard and PirError
        for a partition that refuses (nothing of a refused part is queued)."""
        sid = np.asarray(shard_ids, dtype=np.int64).reshape(-1)
        cid = np.asarray(client_ids, dtype=np.int64).reshape(-1)
        out = np.zeros(sid.size, dtype=TICKET_DTYPE)
        for part, items in sorted(self.router.split(sid).items()):
            pos = np.array([p for p, _ in items], dtype=np.int64)
            local = np.array([s for _, s in items], dtype=np.uint32)
            pcid = np.array([self._clients[int(c)][part] for c in cid[pos]], dtype=np.int32)
            db = self.sdb.dbs[part] if self.sdb is not None else None
            tickets, rc = self.servers[part].submit(db, local, seeds[pos], b_rows[pos], pcid)
            if len(tickets) != pos.size:
                raise RuntimeError(f"partition {part} accepted {len(tickets)} of {pos.size} queries (status {rc})")
            out["part"][pos] = part
            out["ticket"][pos] = tickets
        return out

    def poll_batch(self, tickets: np.ndarray, out: Optional[np.ndarray] = None, timeout_us: int = -1) -> np.ndarray:
        """Collect every ticket (out: (n, 2, plen) uint64, filled in ticket
        order).  Returns out."""
        n = tickets.size
        if out is None:
            out = np.zeros((n, 2, self.sdb.params.plen), dtype=np.uint64)
        for part in np.unique(tickets["part"]):
            pos = np.nonzero(tickets["part"] == part)[0]
            buf = np.zeros((pos.size,) + out.shape[1:], dtype=np.uint64)
            got = self.servers[int(part)].poll_batch(tickets["ticket"][pos], buf, timeout_us)
            if len(got) != pos.size:
                raise TimeoutError(f"partition {int(part)}: {pos.size - len(got)} tickets still pending")
            out[pos] = buf
        return out

    def close(self):
        for s in self.servers:
            s.close()
        self.servers = []


__all__ = ["ShardedDatabase", "MultiGpuServer", "TICKET_DTYPE"]
