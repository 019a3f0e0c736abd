"""Replica partition over GPUs: greedy longest-processing-time (LPT).

Independent replicas (the batched MDPD workload) need no exchange while they
step, so a run on several GPUs gives each rank a set of whole replicas and
gathers only their observables on the host. The cost of a replica's step is
proportional to its particle count, so the replicas are dealt largest first,
each to the rank with the least load so far (Graham's LPT rule: the largest
load is at most 4/3 of the optimum, and at most the mean load plus the
largest single replica).
"""
import heapq


def lpt_partition(sizes, n_ranks):
    """Assigns replica indices to ranks. Returns (parts, loads): parts[k]
    lists rank k's replicas in ascending index order, loads[k] the sum of
    their sizes. Ties go to the lower rank, so the result is deterministic."""
    if n_ranks < 1:
        raise ValueError("n_ranks must be >= 1")
    heap = [(0, k) for k in range(n_ranks)]
    parts = [[] for _ in range(n_ranks)]
    loads = [0] * n_ranks
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    for i in order:
        load, k = heapq.heappop(heap)
        parts[k].append(i)
        loads[k] = load + sizes[i]
        heapq.heappush(heap, (loads[k], k))
    return [sorted(p) for p in parts], loads


def imbalance(loads):
    """Largest load over the mean load (1.0 is perfect balance)."""
    mean = sum(loads) / len(loads)
    return max(loads) / mean if mean > 0 else 1.0
