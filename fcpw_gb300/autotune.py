"""Autotuner of the closest point traversal: times candidate variants
(branching factor, child box precision, and the schedule: a thread per query,
persistent blocks, or warp packets) on a sample of the caller's queries and
keeps the fastest."""
from __future__ import annotations

import itertools

# schedule: "thread" = one thread per query, "persistent" = persistent blocks
# with neighbour seeding, "packet" = the queries of a warp traverse together
DEFAULT_SPACE = {"branching": [2, 4, 8], "bits": [8, 16, 32], "schedule": ["thread", "persistent", "packet"]}


def candidates(space=None, sort_queries=True, precise=True):
    space = dict(space or DEFAULT_SPACE)
    if "schedule" not in space:  # older spelling: a list of persistent flags
        space["schedule"] = ["persistent" if p else "thread" for p in space.get("persistent", [False])]
    for b, q, sch in itertools.product(space["branching"], space["bits"], space["schedule"]):
        yield {"branching": b, "bits": q, "persistent": sch == "persistent", "packet": sch == "packet",
               "sort_queries": sort_queries, "precise": precise}


def autotune_closest_points(gpu, spheres, space=None, reps: int = 3, precise: bool = True, out=None):
    """gpu: GPUScene2D/3D; spheres: (N, 4) float32 CUDA tensor (a representative
    sample). Returns (best config dict, list of (config, ms per call))."""
    import torch
    stream = torch.cuda.current_stream(spheres.device)
    out = out if out is not None else torch.empty((spheres.shape[0], 10), dtype=torch.float32,
                                                  device=spheres.device)
    table = []
    for cfg in candidates(space, precise=precise):
        try:
            gpu.set_traversal(**cfg)
            gpu.find_closest_points_tensor(spheres, out=out)  # builds the wide tree, warms caches
        except Exception:  # a layout this tree cannot be encoded in is skipped
            continue
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(reps):
            gpu.find_closest_points_tensor(spheres, out=out)
        end.record(stream)
        end.synchronize()
        table.append((cfg, start.elapsed_time(end) / reps))
    best = min(table, key=lambda t: t[1])[0]
    gpu.set_traversal(**best)
    return best, table
