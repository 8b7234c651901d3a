"""Lane sharding across GPUs or processes, as the reference partitions cells across arms.

Arm (rank) i of N owns the raw cells pi = i + k*N of its window, starting at cell
i + skip*N and stopping before i + end*N (WZ_FH_SHARD / WZ_FH_NSHARD / WZ_FH_PROF_SKIP /
WZ_FH_PROF_END, src/solver/wz_match.cpp:1573-1586, 2101-2118, 2491-2493). Arms exchange no
data while searching; the global first hit is the minimum over arms of (profile rank, index)
(cluster/deploy/cluster_firsthit_probe.sh:231-236), which global_first_hit() computes with one
all-reduce over the process group after the search.
"""

NO_HIT = (1 << 62)


def owned_cells(ncells, shard, nshard, skip=0, end=0):
    """Raw cell indices the arm visits, in its order."""
    if nshard < 1 or not 0 <= shard < nshard:
        raise ValueError(f"bad shard {shard}/{nshard}")
    stop = min(ncells, shard + end * nshard) if end > 0 else ncells
    return list(range(shard + skip * nshard, stop, nshard))


def global_first_hit(local, group=None):
    """local: (profile_rank, index) of this rank's first hit, or None. Returns the global
    minimum over ranks, or None when no rank found a hit."""
    import torch
    import torch.distributed as dist
    pr, idx = local if local is not None else (NO_HIT, NO_HIT)
    t = torch.tensor([pr, idx], dtype=torch.int64)
    if dist.is_available() and dist.is_initialized():
        # lexicographic min: first the profile rank, then the index among ranks at that rank
        best_pr = t[:1].clone()
        dist.all_reduce(best_pr, op=dist.ReduceOp.MIN, group=group)
        cand = torch.tensor([idx if pr == int(best_pr) else NO_HIT], dtype=torch.int64)
        dist.all_reduce(cand, op=dist.ReduceOp.MIN, group=group)
        pr, idx = int(best_pr), int(cand)
    return None if pr >= NO_HIT else (pr, idx)
