"""Multi-GPU replicas: STA frames are independent (a frame's signal tensor is
read only by that frame's delay-and-sum), so N GPUs run N independent frame
streams with no collective on the data path. These helpers shard frames over
ranks and combine per-rank timings/stats on the host (torch.distributed; NCCL
on GPUs, gloo in the CPU tests)."""
from __future__ import annotations

from typing import Dict, List, Sequence


def shard(num_items: int, rank: int, world: int) -> List[int]:
    """Round-robin assignment of item indices to a rank."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError(f"invalid rank {rank} of {world}")
    return list(range(rank, num_items, world))


def max_over_ranks(value: float, group=None) -> float:
    """Maximum of a per-rank scalar (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(value)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def gather_stats(stats: Dict, group=None) -> List[Dict]:
    """Every rank's stats dict, on every rank."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return [stats]
    out: List = [None] * dist.get_world_size(group)
    dist.all_gather_object(out, stats, group=group)
    return out


def aggregate(per_rank: Sequence[Dict]) -> Dict:
    """Whole-job totals of per-rank frame counts over the slowest rank's time."""
    frames = sum(int(s["frames"]) for s in per_rank)
    seconds = max(float(s["seconds"]) for s in per_rank)
    return {"frames": frames, "seconds": seconds, "frames_per_s": frames / seconds if seconds > 0 else 0.0}
