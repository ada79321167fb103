"""Host-side routing of queries to the GPU that owns their shard.

The Respond path partitions by shard (ShardConfig::index_to_shard,
src/params.rs:553-558): a query reads exactly one shard, so N GPUs each hold a
contiguous range of shards and answer the queries routed to them with no
exchange of data between GPUs.  Throughput over ranks is the total number of
queries divided by the slowest rank's time.
"""
from __future__ import annotations

from dataclasses import dataclass


@dataclass(frozen=True)
class ShardRouter:
    ring_dim: int
    num_shards: int
    world_size: int

    def shards_per_rank(self) -> int:
        return -(-self.num_shards // self.world_size)

    def owner(self, shard_id: int) -> int:
        if not 0 <= shard_id < self.num_shards:
            raise KeyError(f"Shard {shard_id} not found")
        return shard_id // self.shards_per_rank()

    def local_shard(self, shard_id: int) -> int:
        return shard_id - self.owner(shard_id) * self.shards_per_rank()

    def route(self, global_index: int):
        """global entry index -> (rank, local shard id, index within shard)."""
        shard, local = divmod(global_index, self.ring_dim)
        return self.owner(shard), self.local_shard(shard), local

    def split(self, shard_ids):
        """Partition a batch of shard ids by owning rank: {rank: [(pos, local_shard)]}."""
        out: dict[int, list] = {}
        for pos, s in enumerate(shard_ids):
            out.setdefault(self.owner(int(s)), []).append((pos, self.local_shard(int(s))))
        return out


def aggregate_throughput(units: float, seconds: float, group=None) -> float:
    """Total units over all ranks / max seconds over ranks (weak scaling)."""
    import torch
    import torch.distributed as dist

    if group is None and not (dist.is_available() and dist.is_initialized()):
        return units / seconds
    t = torch.tensor([float(units), float(seconds)], dtype=torch.float64)
    u = t[:1].clone()
    s = t[1:].clone()
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(s, op=dist.ReduceOp.MAX, group=group)
    return float(u.item() / s.item())
