"""World-level sharding across GPUs (one process per GPU).

Worlds never read each other's cells, so a set of worlds is split across ranks
with no data exchange at all: every rank computes the same assignment from the
same list of footprints and ticks only its own worlds. Timing is the only thing
the ranks share (a barrier and a max over ranks).
"""


def shard_worlds(footprints, world_size):
    """Assign worlds to ranks by footprint (cells or bytes), largest first, each to
    the currently lightest rank (ties to the lower rank). Deterministic, so every
    rank derives the same shards without communicating. Returns one sorted list of
    world indices per rank; together they partition range(len(footprints))."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(footprints)), key=lambda i: (-int(footprints[i]), i))
    loads = [0] * world_size
    shards = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (loads[k], k))
        shards[r].append(i)
        loads[r] += int(footprints[i])
    return [sorted(s) for s in shards]


def shard_loads(footprints, shards):
    return [sum(int(footprints[i]) for i in s) for s in shards]
