"""Host-side helpers for running the SpMV path on several GPUs of one node.

The single-matrix SpMV runs as independent replicas (one process per GPU,
launched by torchrun): every rank does the same work on its own GPU and the
job's throughput is the units all ranks processed divided by the slowest
rank's time.  A batch of independent matrices shards without any exchange:
each rank takes a subset of the matrices, balanced by nonzeros.
"""
import torch


def max_over_ranks(value, device=None):
    """The maximum of a float over all ranks of the default process group
    (the value itself without one).  `device` is where the reduction tensor
    lives: a CUDA device for NCCL, None (CPU) for gloo."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def shard_matrices(nnz, parts):
    """Greedy balance of matrices over `parts` ranks: matrices in order of
    decreasing nonzeros (ties by index) go to the rank with the fewest
    nonzeros so far (ties by rank).  Deterministic, so every rank computes
    the same assignment.  Returns one sorted list of matrix indices per
    rank."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    order = sorted(range(len(nnz)), key=lambda i: (-int(nnz[i]), i))
    load = [0] * parts
    out = [[] for _ in range(parts)]
    for i in order:
        r = min(range(parts), key=lambda p: (load[p], p))
        out[r].append(i)
        load[r] += int(nnz[i])
    return [sorted(s) for s in out]
