"""Instance shards for several GPUs: the batched workload is a list of independent
propagations, so N GPUs each step their own share of it, with no exchange on the data path
(the only cross-rank work is the timing barrier and a max over ranks).

The shares are balanced by cost = Nr x Ntheta x steps (the grid points each instance moves
through the step's passes), longest processing time first: instances in decreasing cost go
to the currently lightest rank.  Every rank computes the same partition from the same list,
so no rank needs to tell another which instances it took.  The reference steps one
propagation per call (propagation.rs:185-190) and has no multi-device form."""


def instance_cost(params, steps=1):
    """Grid points x steps of one instance (params: a dict with nr and nth)."""
    return int(params["nr"]) * int(params["nth"]) * int(steps)


def partition(costs, world):
    """Indices of the instances on each of `world` ranks: longest processing time first,
    ties broken by instance index (deterministic); each rank's list is in instance order."""
    if world < 1:
        raise ValueError("world must be at least 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def shard(params, world, rank, steps=1):
    """This rank's instances (a sub-list of params, in order) and the whole list's cost."""
    costs = [instance_cost(p, steps) for p in params]
    part = partition(costs, world)[rank]
    return [params[i] for i in part], sum(costs)
