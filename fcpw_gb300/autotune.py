"""Autotuner of the closest point traversal: times candidate variants on a
sample of the caller's queries and keeps the fastest. Stage 1 covers the
branching factor (2/4/8), the child box precision (8/16/32 bits) and the
schedule (a thread per query, persistent blocks, warp packets, or a group
of 2, 4 or 8 lanes per query that splits each record's child boxes and each
leaf's primitives); stage 2
tries merged leaves (subtrees of up to 6, 8 or 12 primitives as one leaf) on
the stage-1 winner; stage 3, for the one-thread-per-query schedules, the
stack placement: 16 entries per thread in shared memory (the default) or the
whole stack in local memory."""
from __future__ import annotations

import itertools

# schedule: "thread" = one thread per query, "persistent" = persistent blocks
# with neighbour seeding, "packet" = the queries of a warp traverse together,
# "packetq" = packets handed to the warps of persistent blocks from a counter,
# "coopL" = L lanes (2, 4, 8) answer one query together
DEFAULT_SPACE = {"branching": [2, 4, 8], "bits": [8, 16, 32],
                 "schedule": ["thread", "persistent", "packet", "packetq", "coop2", "coop4", "coop8"],
                 "leaf_size": [6, 8, 12], "short_stack": [0]}


def lanes_of(schedule: str) -> int:
    return int(schedule[4:]) if schedule.startswith("coop") else 1


def candidates(space=None, sort_queries=True, precise=True):
    """The stage-1 grid (leaf_size 0, short_stack 16)."""
    space = dict(DEFAULT_SPACE, **(space or {}))
    for b, q, sch in itertools.product(space["branching"], space["bits"], space["schedule"]):
        yield {"branching": b, "bits": q, "persistent": sch in ("persistent", "packetq"),
               "packet": sch in ("packet", "packetq"),
               "sort_queries": sort_queries, "precise": precise, "leaf_size": 0, "short_stack": 16,
               "threads_per_query": lanes_of(sch)}


def staged_search(measure, space=None, sort_queries=True, precise=True):
    """measure(cfg) -> ms per call (raises if the layout cannot be encoded).
    Returns (best config, [(config, ms)])."""
    space = dict(DEFAULT_SPACE, **(space or {}))
    table = []

    def run(cfg):
        try:
            table.append((cfg, measure(cfg)))
        except Exception:  # a layout this tree cannot be encoded in is skipped
            pass

    for cfg in candidates(space, sort_queries, precise):
        run(cfg)
    best = min(table, key=lambda t: t[1])[0]
    for leaf in space["leaf_size"]:
        run(dict(best, leaf_size=leaf))
    best = min(table, key=lambda t: t[1])[0]
    if not best["packet"] and best.get("threads_per_query", 1) == 1:
        for short in space["short_stack"]:
            run(dict(best, short_stack=short))
    best = min(table, key=lambda t: t[1])[0]
    return best, table


def autotune_closest_points(gpu, spheres, space=None, reps: int = 3, precise: bool = True, out=None):
    """gpu: GPUScene2D/3D; spheres: (N, 4) float32 CUDA tensor (a representative
    sample). Returns (best config dict, list of (config, ms per call))."""
    import torch
    stream = torch.cuda.current_stream(spheres.device)
    out = out if out is not None else torch.empty((spheres.shape[0], 10), dtype=torch.float32,
                                                  device=spheres.device)

    def measure(cfg):
        gpu.set_traversal(**cfg)
        gpu.find_closest_points_tensor(spheres, out=out)  # builds the wide tree, warms caches
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(reps):
            gpu.find_closest_points_tensor(spheres, out=out)
        end.record(stream)
        end.synchronize()
        return start.elapsed_time(end) / reps

    best, table = staged_search(measure, space, precise=precise)
    gpu.set_traversal(**best)
    return best, table
