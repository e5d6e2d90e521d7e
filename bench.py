"""Benchmark of the closest-point query path on one or more GB300s.

Workload (the 1M-triangle configuration): a seeded torus (R = 1, r = 0.3,
1024 x 512 quads -> 1,048,576 triangles, 2 % radial noise) and 4,194,304 query
points uniform in [-2, 2]^3 with squared max radius = FLT_MAX, binary SAH BVH
built on the host. A step is one closest-point pass over all queries of the
rank, inputs resident on the device; L2 is flushed (a 256 MiB device write)
before every timed step, outside the timed events.

Prints one JSON line (rank 0). ``--impl reference`` instead times the
reference's own CPU implementation (its Scene<3> compiled on this host from its
headers, oracle/_ref; scalar and vectorised builds, the faster one timed) on
all queries of the same workload, with all host threads.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "closest-pt queries/s @1M tris (plain vs batched+quantised, 1 GB300); fwd+bwd ms"
UNIT = "queries/s"
N_QUERIES = 4_194_304
TORUS = (1024, 512)
FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--variant", default="auto")
    ap.add_argument("--queries", type=int, default=N_QUERIES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-loss", action="store_true", help="skip the fwd/fwd+bwd distance loss measurement")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched uneven scenes measurement")
    ap.add_argument("--no-quantised", action="store_true", help="skip the 8/16-bit box measurement")
    ap.add_argument("--no-suite", action="store_true",
                    help="skip the other configurations (icosphere, rays, 2D, 3D silhouettes) in the headline line")
    ap.add_argument("--suite", action="store_true",
                    help="instead of the headline line, one line per other configuration of the scope")
    ap.add_argument("--only", default="",
                    help="with --suite: comma-separated subset of c1,rays,c3,sil3d,inside,instanced,build,batch")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The maximum of x over all ranks (the slowest rank's time); x itself on one rank.
    device: where the reduction tensor lives (the rank's GPU for NCCL, None for gloo)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------- workload
def make_workload(rank: int, n_queries: int):
    """Weak scaling: every rank holds the whole scene and its own query set of
    n_queries (a different seed per rank); no data is exchanged."""
    from fcpw_gb300 import workloads as W
    v, f = W.torus(*TORUS, seed=W.SEED_BASE + 2)
    pts = W.uniform_points(n_queries, 3, -2.0, 2.0, W.SEED_BASE + 2 + 1000 * (rank + 1))
    return v, f, pts


def build_scene(v, f):
    import fcpw_gb300 as F
    s = F.Scene3D()
    s.set_object_count(1)
    s.set_object_vertices(v, 0)
    s.set_object_triangles(f, 0)
    t = time.perf_counter()
    s.build(F.AggregateType.Bvh_SurfaceArea, False)
    return s, time.perf_counter() - t


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling during the timed region (200 ms period)."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- CPU baseline
def reference_cpu(dim, positions, indices, silhouettes=False):
    """The reference's own CPU Scene<DIM> (oracle/_ref, compiled from its headers on this
    host), scalar and, where Enoki builds, vectorised: {"scalar": RefScene, "vectorized":
    RefScene or None}; None when the reference is not available here."""
    from oracle import reference as REF
    if not REF.available():
        return None
    out = {"scalar": REF.RefScene(dim, positions, indices, silhouettes=silhouettes), "vectorized": None}
    if REF.available(simd=True):
        out["vectorized"] = REF.RefScene(dim, positions, indices, silhouettes=silhouettes, vectorize=True)
    return out


def _ref_call(ref_scene, kind, queries, flip=None):
    """One bundled call of the reference's public API; returns the seconds inside it."""
    if kind == "closest":
        return ref_scene.closest_points_timed(queries)[1]
    if kind == "rays":
        return ref_scene.intersect_rays_timed(queries)[1]
    return ref_scene.silhouettes_timed(queries, flip)[1]


def reference_rate(refs, kind, queries, flip=None, budget_s: float = 6.0):
    """Queries/s of the reference CPU on a bounded prefix of `queries` sized to about
    budget_s seconds per build (scalar Bvh and, where it builds, the vectorised Mbvh); the
    faster build is the reported value."""
    threads = os.cpu_count() or 1
    n_all = len(queries)
    rates = {}
    for name in ("scalar", "vectorized"):
        r = refs.get(name)
        if r is None:
            continue
        n0 = min(n_all, 16384)
        sec = _ref_call(r, kind, queries[:n0], None if flip is None else flip[:n0])
        n = int(min(n_all, max(n0, n0 / max(sec, 1e-9) * budget_s)))
        sec = _ref_call(r, kind, queries[:n], None if flip is None else flip[:n])
        rates[name] = (n / sec, n, sec)
    best = max(rates, key=lambda k: rates[k][0])
    v, n, sec = rates[best]
    from oracle import reference as REF
    width = REF.simd_width() if rates.get("vectorized") else 0
    dim = refs[best].dim
    return {"value": v, "unit": UNIT, "cores": threads, "kind": "reference",
            "host": {"cpu": _cpu_model(), "isa": platform.machine()},
            "sample": f"first {n} of {n_all} queries through the reference's Scene<{dim}>::"
                      f"{'findClosestPoints' if kind == 'closest' else ('intersect' if kind == 'rays' else 'findClosestSilhouettePoints')}"
                      f" ({best}{f', FCPW_SIMD_WIDTH={width}' if best == 'vectorized' else ''}), "
                      f"its own std::thread split over {threads} hardware threads, {sec:.2f} s",
            "builds": {k: {"queries_per_s": r[0], "queries": r[1], "seconds": round(r[2], 3)} for k, r in rates.items()}}


def cpu_baseline(v, f, pts, budget_s: float = 12.0):
    """The reference CPU closest-point path (its own compiled Scene<3>, all host threads)
    on a bounded prefix of the query set sized to about budget_s seconds; the oracle's C
    restatement (kind "port") where the reference is not available on this host."""
    from fcpw_gb300 import records as R
    refs = reference_cpu(3, v, f)
    if refs is not None:
        return reference_rate(refs, "closest", R.make_spheres(pts, R.FLT_MAX), budget_s=budget_s / 2)
    return _port_baseline(v, f, pts, budget_s)


def _port_baseline(v, f, pts, budget_s):
    from fcpw_gb300 import records as R
    from oracle import oracle as O
    scene, _ = build_scene(v, f)
    nodes, prims, _ = scene.cpu_bvh.export()
    threads = os.cpu_count() or 1
    n0 = min(len(pts), 20000)
    t = time.perf_counter()
    O.closest_points_bvh(3, nodes, prims, R.make_spheres(pts[:n0], R.FLT_MAX), nthreads=threads)
    rate = n0 / max(time.perf_counter() - t, 1e-9)
    n = int(min(len(pts), max(n0, rate * budget_s)))
    sph = R.make_spheres(pts[:n], R.FLT_MAX)
    t = time.perf_counter()
    O.closest_points_bvh(3, nodes, prims, sph, nthreads=threads)
    dt = time.perf_counter() - t
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {n} of the {len(pts)} queries, oracle/fcpw_oracle.c closest_point_bvh "
                      f"(reference bvh.inl:1291-1418 restated), {threads} threads, {dt:.2f} s"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measure_l2_gbs(dev, reps: int = 50) -> float:
    """Measured L2 throughput of this GPU, for the L2 roofline of the traversal: the best of
    a read (torch sum) and a copy of a 32 MiB float buffer that stays resident in L2,
    CUDA events over `reps` back-to-back calls after warm-up (bytes read + written / time)."""
    import torch
    x = torch.ones(8 << 20, dtype=torch.float32, device=dev)
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream(dev)
    best = 0.0
    for fn, nbytes in ((lambda: x.sum(), x.numel() * 4), (lambda: y.copy_(x), 2 * x.numel() * 4)):
        for _ in range(10):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        b.synchronize()
        best = max(best, nbytes * reps / (a.elapsed_time(b) / 1e3) / 1e9)
    return best


def distance_loss_bench(device_index: int, steps: int = 20, warmup: int = 5):
    """fwd vs fwd+bwd of loss = mean(d^2) on a 200,000-triangle perturbed sphere
    (geodesic frequency 100) and 2^20 uniform queries, with the vertices moved
    onto the device copy and the tree refit on the GPU in every forward."""
    import torch
    import fcpw_gb300 as F
    from fcpw_gb300 import workloads as W
    from fcpw_gb300.autograd import closest_point_distance
    dev = torch.device("cuda", device_index)
    v, f = W.perturbed_sphere(100, W.SEED_BASE + 4)
    s = F.Scene3D()
    s.set_object_count(1)
    s.set_object_vertices(v, 0)
    s.set_object_triangles(f, 0)
    s.build(F.AggregateType.Bvh_SurfaceArea, False)
    gpu = F.GPUScene3D("", False, device=device_index)
    gpu.transfer_to_gpu(s)
    gpu.set_traversal(4, 8, sort_queries=True, persistent=False, precise=True)
    x = torch.from_numpy(W.uniform_points(1 << 20, 3, -1.5, 1.5, W.SEED_BASE + 4)).to(dev)
    verts = torch.from_numpy(v).to(dev).requires_grad_(True)
    stream = torch.cuda.current_stream(dev)

    def fwd():
        d = closest_point_distance(gpu, x, verts, refit=True)
        return (d * d).mean()

    def fwd_bwd():
        verts.grad = None
        fwd().backward()

    def time_it(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / steps

    with torch.no_grad():
        fwd_ms = time_it(fwd)
    fb_ms = time_it(fwd_bwd)
    return {"workload": "loss = mean unsigned distance^2, perturbed sphere 200,000 triangles (geodesic frequency 100), "
                        "2^20 queries uniform in [-1.5,1.5]^3, GPU refit every forward, backward to queries and vertices",
            "fwd_ms": fwd_ms, "fwd_bwd_ms": fb_ms, "ratio": fb_ms / fwd_ms, "target_ratio_max": 2.5}


def algorithmic_bytes(L, g, spheres, out, n, node_bytes, prim_bytes, in_bytes, packet=False):
    """Algorithmic bytes of one closest-point launch, counted by the traversal-statistics
    mode of the same kernel on the same queries (fcpwgb_closest_points_traversal_stats):
    per query in_bytes read and a 40 B record written; per expansion one record of
    node_bytes (the binary kernel loads two 32 B child records per expansion plus the
    root), per primitive test one prim_bytes record; for warp packets one record or
    triangle load serves the 32 queries of a warp."""
    from fcpw_gb300._lib import check
    stats = (C.c_uint64 * 8)()
    check(L.fcpwgb_closest_points_traversal_stats(g.handle, spheres.data_ptr(), out.data_ptr(), n, stats))
    n_q, n_pop, n_inner, n_prim, w_rec, w_prim = [int(x) for x in stats[:6]]
    if node_bytes == 32:
        nb, pb = 32 * (n_q + 2 * n_inner), prim_bytes * n_prim
    elif packet:
        nb, pb = node_bytes * w_rec, prim_bytes * w_prim
    else:
        nb, pb = node_bytes * n_inner, prim_bytes * n_prim
    per_query = {"nodes_popped": n_pop / n_q if node_bytes == 32 else n_inner / n_q,
                 "inner_expanded": n_inner / n_q, "prim_tests": n_prim / n_q}
    # secondary check: about 12 FLOPs per child box test and 60 per primitive test,
    # every expansion testing the record's W child boxes (W = 2 on the binary tree)
    w = int(g.get_traversal()["branching"]) or 2
    per_query["flops_per_query"] = (12 * w * n_inner + 60 * n_prim) / n_q
    if packet:
        per_query.update({"warp_record_loads": w_rec / n_q, "warp_prim_loads": w_prim / n_q})
    return {"bytes": n_q * (in_bytes + 40) + nb + pb, "per_query": per_query}


def run_suite(args):
    for line in suite_records(args, args.only):
        print(json.dumps(line), flush=True)


def per_query_bq(pq, node_bytes, prim_bytes, in_bytes, n, ms, l2_peak):
    """B(q) = in + out + S_record x I(q) + S_prim x P(q) per query (I: records expanded,
    P: primitive tests, both counted for the query itself), summed over the n queries of
    a launch and divided by the kernel time: the L2-served throughput the query stream
    asks for when every query's loads are counted as its own."""
    bq = in_bytes + 40 + node_bytes * pq["inner_expanded"] + prim_bytes * pq["prim_tests"]
    a = bq * n / (ms / 1e3) / 1e9
    return {"bytes_per_query": bq, "achieved": a, "unit": "GB/s", "frac_of_l2_peak": a / l2_peak}


def _compulsory(n, in_b, out_b, scene_bytes, ms, peak):
    """Compulsory-traffic roofline: every query read and every result written once, plus
    the scene's records, over the kernel time, against the HBM peak."""
    b = n * (in_b + out_b) + scene_bytes
    a = b / (ms / 1e3) / 1e9
    return {"bound": "hbm", "compulsory_bytes": int(b), "achieved": a, "peak": peak, "unit": "GB/s",
            "frac": a / peak, "traffic": None}


def suite_records(args, only_arg="", cpu_budget=6.0):
    """One record per configuration of the scope (1M-query icosphere, rays on
    the 1M-triangle torus, 2D segments and silhouettes, 3D silhouettes on the
    torus, and on request contains / line of sight, instances, scene set-up, the
    batch): GPU kernels timed with CUDA events on device-resident inputs (L2
    flushed before each timed call), next to the reference's own CPU Scene
    (its public bundled API, all host threads; the oracle's C restatement where
    the reference is not available) on a bounded sample of the same inputs."""
    import torch
    import fcpw_gb300 as F
    from fcpw_gb300 import records as R
    from fcpw_gb300 import workloads as W
    from fcpw_gb300._lib import check, lib
    from fcpw_gb300.autotune import autotune_closest_points
    from oracle import oracle as O
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    sp = C.c_void_p(stream.cuda_stream)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    L = lib()
    threads = os.cpu_count() or 1

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(reps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            tot += a.elapsed_time(b)
        return tot / reps

    peak, _ = peaks()

    def cpu_rate(fn, n_all, budget_s=cpu_budget):
        n0 = min(n_all, 8192)
        t = time.perf_counter()
        fn(n0)
        rate = n0 / max(time.perf_counter() - t, 1e-9)
        n = int(min(n_all, max(n0, rate * budget_s)))
        t = time.perf_counter()
        fn(n)
        dt = time.perf_counter() - t
        return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port", "sample": f"first {n} of {n_all}"}

    def sph_tensor(pts, r2=R.FLT_MAX):
        t = torch.empty((len(pts), 4), dtype=torch.float32, device=dev)
        t[:, : pts.shape[1]] = torch.from_numpy(pts).to(dev)
        if pts.shape[1] == 2:
            t[:, 2] = 0.0
        t[:, 3] = float(r2)
        return t

    def interior_flips(g, pts):
        """The flip flag of every query as the reference's own tests set it
        (tests/fcpw_tests.py:588-589): 1 for points inside the boundary, from
        the GPU contains batch (equal to Scene::contains bit for bit)."""
        p3 = torch.zeros((len(pts), 3), dtype=torch.float32, device=dev)
        p3[:, : pts.shape[1]] = torch.from_numpy(pts).to(dev)
        flip = g.contains_tensor(p3).to(torch.int32)
        return flip, flip.cpu().numpy().astype(np.uint32)

    def closest_point_config(name, dim, v, idx, pts, silhouettes=False):
        s = F.Scene3D() if dim == 3 else F.Scene2D()
        s.set_object_count(1)
        s.set_object_vertices(v, 0)
        if dim == 3:
            s.set_object_triangles(idx, 0)
        else:
            s.set_object_line_segments(idx, 0)
        if silhouettes:
            s.compute_silhouettes()
        s.build(F.AggregateType.Bvh_SurfaceArea, False)
        g = (F.GPUScene3D if dim == 3 else F.GPUScene2D)("", False, device=0)
        g.transfer_to_gpu(s)
        n = len(pts)
        sph = sph_tensor(pts)
        out = torch.empty((n, 10), dtype=torch.float32, device=dev)

        def run():
            check(L.fcpwgb_find_closest_points_device(g.handle, sph.data_ptr(), out.data_ptr(), n, 0, sp))

        g.set_traversal(0)
        plain_ms = timed(run)
        best, _ = autotune_closest_points(g, sph[: min(n, 1 << 20)])
        fast_ms = timed(run)
        from fcpw_gb300.wide_format import layout
        node_bytes = layout(best["branching"], best["bits"])["size"]
        prim_bytes = 48 if dim == 3 else 24
        alg = algorithmic_bytes(L, g, sph, out, n, node_bytes, prim_bytes, 20, packet=bool(best.get("packet")))
        run()
        k = 1024
        d64 = g.closest_distances_f64_tensor(sph[:k].contiguous()).cpu().numpy()
        rel = np.abs(out[:k, 8].cpu().numpy().astype(np.float64) - d64) / d64
        nodes, prims, sils = s.cpu_bvh.export()
        refs = reference_cpu(dim, v, idx, silhouettes=silhouettes)
        if refs is not None:
            cpu = reference_rate(refs, "closest", R.make_spheres(pts, R.FLT_MAX), budget_s=cpu_budget / 2)
        else:
            cpu = cpu_rate(lambda m: O.closest_points_bvh(dim, nodes, prims, R.make_spheres(pts[:m], R.FLT_MAX),
                                                          nthreads=threads), n)
        roof = _compulsory(n, 16, 40, nodes.nbytes + prims.nbytes, fast_ms, peak)
        a = alg["bytes"] / (fast_ms / 1e3) / 1e9
        roof.update({"algorithmic_bytes": alg["bytes"], "algorithmic_gbs": a, "algorithmic_frac": a / peak,
                     "per_query": alg["per_query"],
                     "time": "CUDA events around the whole call (sort, traversal, refinement)"})
        return s, g, {"config": name, "queries": n, "primitives": int(len(idx)),
                      "plain": {"queries_per_s": n / (plain_ms / 1e3), "ms": plain_ms},
                      "fast": {"queries_per_s": n / (fast_ms / 1e3), "ms": fast_ms, "variant": best},
                      "speedup_vs_plain": plain_ms / fast_ms,
                      "accuracy": {"samples": k, "max_rel_err_vs_fp64": float(rel.max()),
                                   "mean_rel_err_vs_fp64": float(rel.mean())},
                      "roofline": roof, "cpu_baseline": cpu}

    lines = []
    only = set(only_arg.split(",")) if only_arg else None

    def want(name):
        return only is None or name in only

    def sil_run(gs, sph, flip, out, n):
        return lambda: check(L.fcpwgb_find_closest_silhouette_points_device(
            gs.handle, sph.data_ptr(), flip.data_ptr(), out.data_ptr(), n, 0.0, 1e-3, sp))

    def sil_algorithmic(gs, sph, flip, out, n, sil_bytes):
        """Algorithmic bytes of the sorted silhouette packets, counted by their
        statistics mode (fcpwgb_silhouette_traversal_stats) on the same queries:
        per query 16 B sphere, 4 B flag and 4 B sort index read, 40 B record written;
        per warp step the current node's 32 B box part, plus two 64 B child records at
        an inner node or the node's 32 B cone part and its silhouette records at a leaf."""
        gs.set_traversal(4, 32, sort_queries=True)
        st = (C.c_uint64 * 8)()
        check(L.fcpwgb_silhouette_traversal_stats(gs.handle, sph.data_ptr(), flip.data_ptr(), out.data_ptr(), n,
                                                  C.c_float(0.0), C.c_float(1e-3), st))
        gs.set_traversal(0)
        n_q, w_in, w_leaf, w_sil, t_child, t_sil = [int(x) for x in st[:6]]
        b = n_q * (24 + 40) + w_in * (32 + 128) + w_leaf * (32 + 32) + w_sil * sil_bytes
        return b, {"warp_inner_steps": w_in / n_q, "warp_leaf_steps": w_leaf / n_q, "warp_sil_loads": w_sil / n_q,
                   "child_tests": t_child / n_q, "sil_tests": t_sil / n_q}

    def sil_times(gs, sph, flip, out, n):
        gs.set_traversal(0)
        plain = timed(sil_run(gs, sph, flip, out, n))
        variants = {}
        # a fast-path configuration: warp packets on the binary SNCH tree (k_sil_packet.cu)
        for sort in (True, False):
            gs.set_traversal(4, 32, sort_queries=sort)
            variants["warp packets, queries sorted" if sort else "warp packets, caller order"] = timed(
                sil_run(gs, sph, flip, out, n))
        gs.set_traversal(0)
        best = min(variants, key=variants.get)
        fast = variants[best]
        return {"plain": {"queries_per_s": n / (plain / 1e3), "ms": plain},
                "fast": {"queries_per_s": n / (fast / 1e3), "ms": fast, "variant": best},
                "variants_ms": {k: round(v, 3) for k, v in variants.items()},
                "speedup_vs_plain": plain / fast}

    def sil_roofline(gs, sph, flip, out, n, times, scene_bytes, sil_bytes):
        roof = _compulsory(n, 20, 40, scene_bytes, times["fast"]["ms"], peak)
        ab, per_q = sil_algorithmic(gs, sph, flip, out, n, sil_bytes)
        a = ab / (times["variants_ms"]["warp packets, queries sorted"] / 1e3) / 1e9
        roof.update({"algorithmic_bytes": ab, "algorithmic_gbs": a, "algorithmic_frac": a / peak, "per_query": per_q,
                     "time": "CUDA events around the whole call (sort, packets)"})
        return roof

    # C1: 20,480-triangle perturbed icosphere, 1,048,576 queries in [-1.5, 1.5]^3
    if want("c1"):
        v, f = W.perturbed_sphere(32, W.SEED_BASE + 1)
        _, _, line = closest_point_config("icosphere 20,480 triangles, 1,048,576 closest-point queries", 3, v, f,
                                          W.uniform_points(1 << 20, 3, -1.5, 1.5, W.SEED_BASE + 1001))
        lines.append(line)

    # C2 rays: 4,194,304 rays on the 1M-triangle torus, origins in [-2, 2]^3, directions uniform on S^2
    if want("rays"):
        v, f, _ = make_workload(0, 1)
        s, _ = build_scene(v, f)
        g = F.GPUScene3D("", False, device=0)
        g.transfer_to_gpu(s)
        n = N_QUERIES
        o = W.uniform_points(n, 3, -2.0, 2.0, W.SEED_BASE + 2002)
        d = W.uniform_directions(n, 3, W.SEED_BASE + 2003)
        rays_np = R.make_rays(o, d, R.FLT_MAX)
        rays = torch.from_numpy(rays_np.view(np.float32).reshape(n, 10).copy()).to(dev)
        out = torch.empty((n, 10), dtype=torch.float32, device=dev)
        def ray_run():
            check(L.fcpwgb_intersect_rays_device(g.handle, rays.data_ptr(), out.data_ptr(), n, 0, sp))

        g.set_traversal(0)
        ray_ms = timed(ray_run)
        hits = float((out[:, 9].view(torch.int32) != -1).float().mean())
        table = []
        # (branching, bits, sort, schedule): 0 one thread per ray, 1 warp packets, 2 per-lane refill
        # (the refill schedule reads the caller's order: no sort)
        for wb in [(2, 32, True, 0), (4, 8, True, 0), (4, 16, True, 0), (4, 32, True, 0), (4, 32, False, 0),
                   (8, 8, True, 0), (8, 16, True, 0), (8, 32, True, 0), (4, 32, True, 1), (8, 32, True, 1),
                   (2, 32, False, 2), (4, 8, False, 2), (4, 16, False, 2), (4, 32, False, 2), (8, 8, False, 2),
                   (8, 16, False, 2), (8, 32, False, 2)]:
            g.set_traversal(*wb[:2], sort_queries=wb[2], packet=wb[3] == 1, persistent=wb[3] == 2)
            table.append((wb, timed(ray_run, reps=3)))
        (wb_best, _) = min(table, key=lambda t: t[1])
        g.set_traversal(*wb_best[:2], sort_queries=wb_best[2], packet=wb_best[3] == 1, persistent=wb_best[3] == 2)
        fast_ms = timed(ray_run)
        nodes, prims, _ = s.cpu_bvh.export()
        refs = reference_cpu(3, v, f)
        if refs is not None:
            cpu = reference_rate(refs, "rays", rays_np, budget_s=cpu_budget / 2)
        else:
            cpu = cpu_rate(lambda m: O.intersect_rays_bvh(3, nodes, prims, rays_np[:m], nthreads=threads), n)
        del refs
        # FP64 hit parameter of the triangle each of 1024 rays hit (the plane through its vertices)
        res = out[:1024].cpu().numpy().view(R.INTERACTION).reshape(-1)
        hk = np.nonzero(res["index"] != R.UINT_MAX)[0]
        pos = np.empty(len(prims), np.int64)
        pos[prims["index"].astype(np.int64)] = np.arange(len(prims))
        pk = pos[res["index"][hk].astype(np.int64)]
        a, b, c = (prims[x][pk].astype(np.float64) for x in ("pa", "pb", "pc"))
        nrm = np.cross(b - a, c - a)
        ro, rd = o[hk].astype(np.float64), d[hk].astype(np.float64)
        t64 = np.einsum("ij,ij->i", nrm, a - ro) / np.einsum("ij,ij->i", nrm, rd)
        rel_t = np.abs(res["d"][hk].astype(np.float64) - t64) / t64
        lines.append({"config": "rays, torus 1,048,576 triangles, 4,194,304 rays (first hit)", "queries": n,
                      "accuracy": {"samples": int(len(hk)), "max_rel_err_vs_fp64": float(rel_t.max()),
                                   "mean_rel_err_vs_fp64": float(rel_t.mean()),
                                   "what": "hit distance against the FP64 plane parameter of the same triangle"},
                      "roofline": _compulsory(n, 40, 40, nodes.nbytes + prims.nbytes, fast_ms, peak),
                      "plain": {"queries_per_s": n / (ray_ms / 1e3), "ms": ray_ms},
                      "fast": {"queries_per_s": n / (fast_ms / 1e3), "ms": fast_ms,
                               "variant": {"branching": wb_best[0], "bits": wb_best[1], "sort_queries": wb_best[2],
                                           "schedule": ["thread", "packet", "refill"][wb_best[3]]}},
                      "speedup_vs_plain": ray_ms / fast_ms, "hit_fraction": hits,
                      "autotune_ms": [[w, b, int(o), ["thread", "packet", "refill"][pk], round(t, 3)]
                                      for (w, b, o, pk), t in table],
                      "cpu_baseline": cpu})
        del g, s

    # C3: 256 star polylines x 512 segments, 8,388,608 queries in [-3, 3]^2: closest point and silhouettes
    if want("c3"):
        v, sg = W.star_polylines(256, 512, W.SEED_BASE + 3, extent=3.0, scale=0.14)
        pts2 = W.uniform_points(8 << 20, 2, -3.0, 3.0, W.SEED_BASE + 3003)
        s2, g2, line = closest_point_config("2D stars 131,072 segments, 8,388,608 closest-point queries", 2, v, sg,
                                            pts2, silhouettes=True)
        lines.append(line)
        n = len(pts2)
        sph = sph_tensor(pts2)
        g2.set_traversal(0)
        flip, hflip = interior_flips(g2, pts2)
        out = torch.empty((n, 10), dtype=torch.float32, device=dev)
        times = sil_times(g2, sph, flip, out, n)
        nodes, _, sils = s2.cpu_bvh.export()
        refs = reference_cpu(2, v, sg, silhouettes=True)
        if refs is not None:
            cpu = reference_rate(refs, "silhouettes", R.make_spheres(pts2, R.FLT_MAX), flip=hflip,
                                 budget_s=cpu_budget / 2)
        else:
            cpu = cpu_rate(lambda m: O.silhouettes_bvh(2, nodes, sils, R.make_spheres(pts2[:m], R.FLT_MAX),
                                                       hflip[:m], nthreads=threads), n)
        del refs
        lines.append({"config": "2D stars 131,072 segments, 8,388,608 closest-silhouette queries "
                                f"(flip 1 inside the boundary: {int(hflip.sum()):,} queries)",
                      "queries": n, **times,
                      "roofline": sil_roofline(g2, sph, flip, out, n, times, nodes.nbytes + sils.nbytes, 32),
                      "accuracy": "no FP64 silhouette oracle; parity with the reference's answers is tested",
                      "cpu_baseline": cpu})
        del g2, s2

    # 3D silhouettes (SNCH) on the 1M-triangle torus, 4,194,304 queries in [-2, 2]^3, and on the
    # 20,480-triangle icosphere with its 1,048,576 queries in [-1.5, 1.5]^3
    if want("sil3d"):
        v, f, pts = make_workload(0, args.queries)
        vi, fi = W.perturbed_sphere(32, W.SEED_BASE + 1)
        pts_i = W.uniform_points(1 << 20, 3, -1.5, 1.5, W.SEED_BASE + 1001)
        for mesh, (vv, ff, pp) in (("torus 1,048,576 triangles", (v, f, pts)),
                                   ("icosphere 20,480 triangles", (vi, fi, pts_i))):
            s = F.Scene3D()
            s.set_object_count(1)
            s.set_object_vertices(vv, 0)
            s.set_object_triangles(ff, 0)
            s.compute_silhouettes()
            s.build(F.AggregateType.Bvh_SurfaceArea, False)
            g = F.GPUScene3D("", False, device=0)
            g.transfer_to_gpu(s)
            n = len(pp)
            sph = sph_tensor(pp)
            g.set_traversal(0)
            flip, hflip = interior_flips(g, pp)
            out = torch.empty((n, 10), dtype=torch.float32, device=dev)
            times = sil_times(g, sph, flip, out, n)
            nodes, _, sils = s.cpu_bvh.export()
            cpu = None
            if not args.no_cpu_baseline:
                refs = reference_cpu(3, vv, ff, silhouettes=True)
                if refs is not None:
                    cpu = reference_rate(refs, "silhouettes", R.make_spheres(pp, R.FLT_MAX), flip=hflip,
                                         budget_s=cpu_budget / 2)
                else:
                    cpu = cpu_rate(lambda m: O.silhouettes_bvh(3, nodes, sils, R.make_spheres(pp[:m], R.FLT_MAX),
                                                               hflip[:m], nthreads=threads), n)
                del refs
            lines.append({"config": f"3D silhouettes, {mesh} (SNCH), {n:,} queries "
                                    f"(flip 1 inside the boundary: {int(hflip.sum()):,} queries)",
                          "queries": n, **times,
                          "roofline": sil_roofline(g, sph, flip, out, n, times, nodes.nbytes + sils.nbytes, 56),
                          "accuracy": "no FP64 silhouette oracle; parity with the reference's answers is tested",
                          "cpu_baseline": cpu})
            del g, s

    # contains / line of sight (CPU-only in the reference) on the 1M-triangle torus
    if want("inside"):
        v, f, pts = make_workload(0, N_QUERIES)
        s, _ = build_scene(v, f)
        g = F.GPUScene3D("", False, device=0)
        g.transfer_to_gpu(s)
        n = len(pts)
        pb = W.uniform_points(n, 3, -2.0, 2.0, W.SEED_BASE + 4004)
        ta = torch.from_numpy(pts).to(dev)
        tb = torch.from_numpy(pb).to(dev)
        res = torch.empty(n, dtype=torch.int32, device=dev)
        g.set_traversal(0)  # the caller's order
        in_plain_ms = timed(lambda: g.contains_tensor(ta, out=res))
        g.set_traversal(4, 32, sort_queries=True)  # points sorted spatially first, same answers
        in_ms = timed(lambda: g.contains_tensor(ta, out=res))
        inside = float(res.float().mean())
        g.set_traversal(0)
        los_ms = timed(lambda: g.has_line_of_sight_tensor(ta, tb, out=res))
        visible = float(res.float().mean())
        nodes, prims, _ = s.cpu_bvh.export()
        cpu_in = cpu_rate(lambda m: O.contains_bvh(3, nodes, prims, pts[:m], nthreads=threads), n)
        cpu_los = cpu_rate(lambda m: O.line_of_sight_bvh(3, nodes, prims, pts[:m], pb[:m], nthreads=threads), n)
        lines.append({"config": "contains, torus 1,048,576 triangles, 4,194,304 points (two all-hits rays each)",
                      "queries": n, "gpu": {"queries_per_s": n / (in_ms / 1e3), "ms": in_ms,
                                            "variant": "points sorted spatially"},
                      "caller_order": {"queries_per_s": n / (in_plain_ms / 1e3), "ms": in_plain_ms},
                      "inside_fraction": inside, "cpu_baseline": cpu_in})
        lines.append({"config": "line of sight, torus 1,048,576 triangles, 4,194,304 point pairs", "queries": n,
                      "gpu": {"queries_per_s": n / (los_ms / 1e3), "ms": los_ms}, "visible_fraction": visible,
                      "cpu_baseline": cpu_los})

    # several objects with instance transforms: 64 rotated and scaled copies of a 65,536-triangle torus,
    # 64 of a 20,480-triangle sphere and one untransformed sphere, 4,194,304 queries in [-8, 8]^3
    if want("instanced"):
        rng = np.random.default_rng(W.SEED_BASE + 5005)

        def affines(k):
            out_m = []
            for _ in range(k):
                a = rng.normal(size=3)
                a /= np.linalg.norm(a)
                ang = rng.uniform(0, 2 * np.pi)
                kk = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
                rot = np.eye(3) * np.cos(ang) + np.sin(ang) * kk + (1 - np.cos(ang)) * np.outer(a, a)
                m = np.eye(4)
                m[:3, :3] = rot * rng.uniform(0.3, 1.0)
                m[:3, 3] = rng.uniform(-7.0, 7.0, 3)
                out_m.append(m.astype(np.float32))
            return out_m

        vt, ft = W.torus(256, 128, W.SEED_BASE + 5006)
        vs, fs = W.perturbed_sphere(32, W.SEED_BASE + 5007)
        s = F.Scene3D()
        s.set_object_count(3)
        for k, (v, f) in enumerate([(vt, ft), (vs, fs), (vs, fs)]):
            s.set_object_vertices(v, k)
            s.set_object_triangles(f, k)
        s.set_object_instance_transforms(affines(64), 0)
        s.set_object_instance_transforms(affines(64), 1)
        s.build(F.AggregateType.Bvh_SurfaceArea, False)
        n = N_QUERIES
        pts = W.uniform_points(n, 3, -8.0, 8.0, W.SEED_BASE + 5008)
        sph = sph_tensor(pts)
        out = torch.empty((n, 10), dtype=torch.float32, device=dev)
        inst_out = torch.empty(n, dtype=torch.int32, device=dev)
        g = F.GPUScene3D("", False, device=0)
        g.transfer_to_gpu(s)

        def inst_run():
            check(L.fcpwgb_find_closest_points_instanced_device(g.handle, sph.data_ptr(), out.data_ptr(),
                                                                inst_out.data_ptr(), n, 0, sp))

        table = {}
        for bits in (32, 16, 8):
            g.set_traversal(4, bits, sort_queries=True)
            table[bits] = timed(inst_run)
        best_bits = min(table, key=table.get)
        inst = s.instances
        top_nodes, top_refs, mats = inst.export()
        objs = [o.export()[:2] for o in inst.objects]
        cpu = cpu_rate(lambda m: O.instanced_closest_points(3, top_nodes, top_refs, mats, inst.instance_objects,
                                                            inst.transformed, objs,
                                                            R.make_spheres(pts[:m], R.FLT_MAX), nthreads=threads),
                       n)
        world_tris = 64 * len(ft) + 65 * len(fs)
        lines.append({"config": f"instanced: 129 instances of 3 objects ({world_tris:,} triangles in world space), "
                                f"{n:,} closest-point queries", "queries": n, "instances": len(inst),
                      "gpu": {"queries_per_s": n / (table[best_bits] / 1e3), "ms": table[best_bits],
                              "variant": {"branching": 4, "bits": best_bits, "sort_queries": True}},
                      "ms_by_bits": {str(b): round(t, 3) for b, t in table.items()}, "cpu_baseline": cpu})
        del g, s

    # scene setup on the 1M-triangle torus: the host SAH build (the reference's algorithm) and its
    # transfer against the GPU build with its transfer
    if want("build"):
        v, f, _ = make_workload(0, 1)
        t0 = time.perf_counter()
        s, _ = build_scene(v, f)
        t_host = time.perf_counter() - t0
        g = F.GPUScene3D("", False, device=0)
        t0 = time.perf_counter()
        g.transfer_to_gpu(s)
        torch.cuda.synchronize()
        t_transfer = time.perf_counter() - t0
        vd, fd = torch.from_numpy(v).to(dev), torch.from_numpy(f).to(dev)

        def gpu_build(method):
            gb = F.GPUScene3D("", False, device=0)
            gb.build_on_gpu(vd, fd, method=method)
            runs = []
            for _ in range(3):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                gb.build_on_gpu(vd, fd, method=method)
                torch.cuda.synchronize()
                runs.append(time.perf_counter() - t0)
            return gb, min(runs)

        gl, t_lbvh = gpu_build("lbvh")
        gs, t_sah = gpu_build("sah")
        same = bool(np.array_equal(gs.export_nodes().view(np.uint8), g.export_nodes().view(np.uint8)))
        lines.append({"config": f"scene setup, torus {len(f):,} triangles", "host_sah_build_s": t_host,
                      "host_transfer_s": t_transfer,
                      "gpu_sah_build_and_transfer_s": t_sah, "gpu_sah_tree_equals_host": same,
                      "speedup_sah": (t_host + t_transfer) / t_sah,
                      "gpu_lbvh_build_and_transfer_s": t_lbvh, "speedup_lbvh": (t_host + t_transfer) / t_lbvh,
                      "host_tree_nodes": g.info()["n_nodes"], "lbvh_tree_nodes": gl.info()["n_nodes"]})
        del g, gl, gs, s

    # the 512-mesh batch alone (also part of the headline line)
    if want("batch") and only is not None:
        lines.append({"config": "batched uneven scenes", **batched_scenes_bench(0)})

    return lines


def _schedule(c) -> str:
    lanes = c.get("threads_per_query", 1)
    s = ("packetq" if c.get("persistent") else "packet") if c.get("packet") else \
        (f"coop{lanes}" if lanes > 1 else ("persistent" if c.get("persistent") else "thread"))
    if c.get("leaf_size"):
        s += f"+leaf{c['leaf_size']}"
    if not c.get("packet") and lanes == 1 and c.get("short_stack", 16) != 16:
        s += f"+stack{c['short_stack']}"
    return s


def batched_scenes_bench(device_index: int, reps: int = 5):
    """Batched uneven scenes: 512 seeded meshes (perturbed geodesic spheres and
    tori, triangle counts log-uniform in [1e3, 2e5], queries per mesh
    log-uniform in [1e3, 1e6]) answered by one persistent launch over the
    forest, replayed from a captured CUDA graph, with branching and box
    precision autotuned. Compared with one GPUScene per mesh and one launch per
    mesh: the plain binary kernel, and the same wide variant."""
    import concurrent.futures
    import torch
    import fcpw_gb300 as F
    from fcpw_gb300 import records as R
    from fcpw_gb300 import workloads as W
    from fcpw_gb300._lib import check, lib
    from fcpw_gb300.batch import autotune_batch
    dev = torch.device("cuda", device_index)
    t0 = time.perf_counter()
    meshes, counts, boxes = W.batched_meshes()
    pts = W.batched_queries(counts, boxes, W.SEED_BASE + 6)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(os.cpu_count() or 1) as ex:  # the native build releases the GIL
        scenes = list(ex.map(lambda m: build_scene(*m)[0], meshes))
    build_s = time.perf_counter() - t0
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    n = int(offsets[-1])
    spheres = torch.empty((n, 4), dtype=torch.float32, device=dev)
    spheres[:, :3] = torch.from_numpy(pts).to(dev)
    spheres[:, 3] = float(R.FLT_MAX)
    del pts
    out = torch.empty((n, 10), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    batch = F.GPUSceneBatch3D(device_index)
    t0 = time.perf_counter()
    batch.set_scenes(scenes)
    set_s = time.perf_counter() - t0
    space = {"branching": [2, 4, 8], "bits": [8, 16, 32], "schedule": ["thread", "packet", "packetq"],
             "leaf_size": [8], "short_stack": [0]}
    best, table = autotune_batch(batch, spheres, offsets, space=space, reps=2)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / reps

    ms = timed(lambda: batch.find_closest_points_tensor(spheres, offsets, out=out))
    stats = batch.traversal_stats(spheres, offsets, out)
    info = batch.info()
    res = out.clone()

    # one scene and one launch per mesh
    gpus = []
    for s in scenes:
        g = F.GPUScene3D("", False, device=device_index)
        g.transfer_to_gpu(s)
        gpus.append(g)
    L = lib()
    sp = C.c_void_p(stream.cuda_stream)

    def per_scene():
        for k, g in enumerate(gpus):
            a, m = int(offsets[k]), int(counts[k])
            check(L.fcpwgb_find_closest_points_device(g.handle, spheres[a:].data_ptr(), out[a:].data_ptr(), m, 0, sp))

    for g in gpus:
        g.set_traversal(0)
    plain_ms = timed(per_scene)
    for g in gpus:
        g.set_traversal(best["branching"], best["bits"], sort_queries=True, persistent=False, precise=True,
                        packet=best.get("packet", False), leaf_size=best.get("leaf_size", 0),
                        short_stack=best.get("short_stack", 16))
    wide_ms = timed(per_scene)

    # FP64 error of the batched results on 256 queries of each of 8 scenes
    rel = []
    for k in np.linspace(0, len(scenes) - 1, 8).astype(int):
        a, m = int(offsets[k]), min(int(counts[k]), 256)
        d64 = gpus[k].closest_distances_f64_tensor(spheres[a:a + m].contiguous()).cpu().numpy()
        d = res[a:a + m, 8].cpu().numpy().astype(np.float64)
        rel.append(np.abs(d - d64) / d64)
    rel = np.concatenate(rel)
    del gpus
    return {"workload": "512 meshes (perturbed geodesic spheres / tori 50:50, triangles log-uniform in [1e3, 2e5], "
                        "queries per mesh log-uniform in [1e3, 1e6], uniform in each mesh's cube grown by 25 %), "
                        "r2 = FLT_MAX; one graph launch per batch (sort + persistent-capable wide traversal)",
            "meshes": len(scenes), "triangles": info["primitives"], "queries": n,
            "queries_per_s": n / (ms / 1e3), "ms": ms, "variant": best,
            "autotune_ms": [[c["branching"], c["bits"], _schedule(c), round(t, 3)] for c, t in table],
            "per_query": {"wide_records_expanded": stats["expanded"] / n, "prim_tests": stats["prim_tests"] / n},
            "per_scene_plain": {"variant": "one GPUScene and one launch per mesh, binary tree, reference order",
                                "queries_per_s": n / (plain_ms / 1e3), "ms": plain_ms},
            "per_scene_wide": {"variant": "one GPUScene and one launch per mesh, same wide variant",
                               "queries_per_s": n / (wide_ms / 1e3), "ms": wide_ms},
            "speedup_vs_per_scene_plain": plain_ms / ms,
            "accuracy": {"samples": int(len(rel)), "max_rel_err_vs_fp64": float(rel.max()),
                         "mean_rel_err_vs_fp64": float(rel.mean())},
            "l2": "inputs (1 GB queries, 2.4 GB results) exceed L2; no flush",
            "setup_s": {"generate": round(gen_s, 2), "bvh_builds": round(build_s, 2), "set_scenes": round(set_s, 2)}}


# ------------------------------------------------------------------ main
def run_ours(args):
    import torch
    import torch.distributed as dist
    import fcpw_gb300 as F
    from fcpw_gb300 import records as R
    from fcpw_gb300._lib import check, lib
    from fcpw_gb300.autotune import autotune_closest_points

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    v, f, pts = make_workload(rank, args.queries)
    scene, build_s = build_scene(v, f)
    gpu = F.GPUScene3D("", False, device=local)
    t = time.perf_counter()
    gpu.transfer_to_gpu(scene)
    transfer_s = time.perf_counter() - t
    n = len(pts)

    spheres = torch.empty((n, 4), dtype=torch.float32, device=dev)
    spheres[:, :3] = torch.from_numpy(pts).to(dev)
    spheres[:, 3] = float(R.FLT_MAX)
    out = torch.empty((n, 10), dtype=torch.float32, device=dev)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = C.c_void_p(stream.cuda_stream)
    L = lib()

    def step():
        check(L.fcpwgb_find_closest_points_device(gpu.handle, spheres.data_ptr(), out.data_ptr(), n, 0, sptr))

    def traversal_stats(node_bytes, prim_bytes, in_bytes, packet=False):
        return algorithmic_bytes(L, gpu, spheres, out, n, node_bytes, prim_bytes, in_bytes, packet)

    def timed(steps, warmup):
        for _ in range(warmup):
            flush.zero_()
            step()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        check(L.fcpwgb_gpu_scene_enable_kernel_timing(gpu.handle, 1))
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        for i in range(steps):
            flush.zero_()
            starts[i].record(stream)
            step()
            ends[i].record(stream)
        torch.cuda.synchronize()
        ktot, kn = C.c_double(0), C.c_uint32(0)
        check(L.fcpwgb_gpu_scene_kernel_time(gpu.handle, C.byref(ktot), C.byref(kn)))
        check(L.fcpwgb_gpu_scene_enable_kernel_timing(gpu.handle, 0))
        if world > 1:
            dist.barrier()
        ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / steps
        return ms, ktot.value / max(kn.value, 1)

    # 1) plain: the binary tree in the reference GPU traversal order
    gpu.set_traversal(0)
    plain_ms, plain_kms = timed(max(3, args.steps // 4), 2)
    plain_stats = traversal_stats(32, 40, 16)

    # 2) fast path: wide tree with quantised child boxes, queries sorted, persistent blocks, refined final distance
    sample = spheres[: min(n, 1 << 20)]
    if args.variant == "auto":
        best, table = autotune_closest_points(gpu, sample)
    else:  # fixed "branching,bits,schedule" (0 thread, 1 persistent, 2 packet, 3/4/5 groups of 2/4/8 lanes,
        # 6 packets from a counter), e.g. for profiling one kernel
        b, q, p = (int(x) for x in args.variant.split(","))
        best = {"branching": b, "bits": q, "persistent": p in (1, 6), "packet": p in (2, 6), "sort_queries": True,
                "precise": True, "threads_per_query": {3: 2, 4: 4, 5: 8}.get(p, 1)}
        gpu.set_traversal(**best)
        table = []
    from fcpw_gb300.wide_format import layout
    node_bytes = layout(best["branching"], best["bits"])["size"]
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    ms, kms = timed(args.steps, args.warmup)
    fast_stats = traversal_stats(node_bytes, 48, 20, packet=bool(best.get("packet")))  # sorted query + permutation
    ms_max = max_over_ranks(ms, world, dev)
    value = world * n / (ms_max / 1e3)

    # quantised child boxes: the best 4- or 8-wide, one-thread or packet variant per precision, all queries
    quantised = {}
    if args.variant == "auto" and not args.no_quantised:
        for bits in (8, 16):
            rows = []
            for br in (4, 8):
                for sch in ("thread", "packet", "packetq"):
                    cfg = dict(best, branching=br, bits=bits, persistent=sch == "packetq", packet=sch != "thread",
                               leaf_size=0, short_stack=16, threads_per_query=1)
                    try:
                        gpu.set_traversal(**cfg)
                        rows.append((cfg, timed(3, 2)[0]))
                    except Exception:  # a layout this tree cannot be encoded in is skipped
                        pass
            if rows:
                cfg, qms = min(rows, key=lambda t: t[1])
                gpu.set_traversal(**cfg)
                step()
                d64q = gpu.closest_distances_f64_tensor(spheres[:1024]).cpu().numpy()
                relq = np.abs(out[:1024, 8].cpu().numpy().astype(np.float64) - d64q) / d64q
                quantised[f"q{bits}"] = {
                    "variant": f"wide{cfg['branching']}_q{bits}_" + _schedule(cfg),
                    "queries_per_s": world * n / (qms / 1e3), "ms_per_step": qms,
                    "speedup_vs_plain": plain_ms / qms, "vs_float_boxes": ms / qms,
                    "accuracy": {"samples": 1024, "max_rel_err_vs_fp64": float(relq.max()),
                                 "mean_rel_err_vs_fp64": float(relq.mean())},
                    "all_ms": {f"wide{c['branching']}_q{bits}_" + _schedule(c): round(t, 3) for c, t in rows}}
        gpu.set_traversal(**best)

    # end to end through the host-array C ABI call (pinned host buffers, copies inside)
    h_sph = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
    h_sph.copy_(spheres.cpu())
    h_out = torch.empty((n, 10), dtype=torch.float32, pin_memory=True)
    for _ in range(2):
        check(L.fcpwgb_find_closest_points(gpu.handle, h_sph.data_ptr(), h_out.data_ptr(), n, 0))
    e2e_t = []
    for _ in range(max(3, args.steps // 2)):
        t = time.perf_counter()
        check(L.fcpwgb_find_closest_points(gpu.handle, h_sph.data_ptr(), h_out.data_ptr(), n, 0))
        e2e_t.append(time.perf_counter() - t)
    clocks = sampler.stop()
    e2e_s = statistics.median(e2e_t)
    e2e_value = world * n / max_over_ranks(e2e_s, world, dev)

    result = None
    if rank == 0:
        res = h_out.numpy().view(R.INTERACTION).reshape(-1)
        k = 1024  # FP64 brute force over all triangles on the GPU (fcpwgb_closest_distances_f64_device)
        d64 = gpu.closest_distances_f64_tensor(spheres[:k]).cpu().numpy()
        rel = np.abs(res["d"][:k].astype(np.float64) - d64) / d64
        accuracy = {"samples": k, "max_rel_err_vs_fp64": float(rel.max()), "mean_rel_err_vs_fp64": float(rel.mean()),
                    "variant": "fast path (precise)"}

        peak, peak_kind = peaks()
        achieved = fast_stats["bytes"] / (kms / 1e3) / 1e9
        variant = f"wide{best['branching']}_q{best['bits']}_" + _schedule(best)
        l2_peak = measure_l2_gbs(dev)
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded torus + uniform queries)",
            "config": {"workload": "closest point, seeded torus 1,048,576 triangles, 4,194,304 queries "
                                   "uniform in [-2,2]^3 per GPU, r2 = FLT_MAX, SAH BVH",
                       "variant": variant, "traversal": best, "queries_per_gpu": n, "triangles": int(len(f)),
                       "l2": "flushed (256 MiB write) before every timed step",
                       "bvh_build_s": round(build_s, 3), "transfer_s": round(transfer_s, 3),
                       "plain": {"variant": "binary tree, reference traversal order (bvh.slang:395-502)",
                                 "queries_per_s": world * n / (plain_ms / 1e3), "ms_per_step": plain_ms,
                                 "kernel_ms": plain_kms, "per_query": plain_stats["per_query"],
                                 "achieved_gbs": plain_stats["bytes"] / (plain_kms / 1e3) / 1e9},
                       "speedup_vs_plain": plain_ms / ms,
                       "autotune_ms": [[c["branching"], c["bits"], _schedule(c), round(t, 4)]
                                       for c, t in table]},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 16, "d2h_bytes_per_step": n * 40},
            # per timed step: the query-bound reduction, histogram, three scan kernels and the scatter of
            # the spatial sort (when on), then the traversal kernel and the precise mode's refinement pass
            "gpu_launches": args.steps * ((7 if best.get("sort_queries", True) else 1) + 1),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": f"hbm_gbs ({peak_kind})",
                         "kernel": ("kWidePacketClosestPoint" if best.get("packet") else "kWideClosestPoint")
                         + " + kRefineClosest",
                         "kernel_ms": kms,  # CUDA events around both kernels of the precise launch
                         "algorithmic_bytes_per_launch": fast_stats["bytes"], "per_query": fast_stats["per_query"],
                         # the records and triangles (24-57 MB) stay in L2, so the loads counted above are
                         # served by L2: the ceiling that applies is L2 throughput and instruction issue
                         "l2": {"achieved": achieved, "peak": l2_peak, "unit": "GB/s", "frac": achieved / l2_peak,
                                "peak_source": "measured in this run: best of a read and a copy of a 32 MiB "
                                               "L2-resident buffer"},
                         # the per-query B(q) of the scope's definition: every query's own expansions and
                         # tests counted as its own record and triangle loads; the warp packets serve each
                         # load to all lanes that need it, so this exceeds what the memory system moves
                         "per_query_bq": per_query_bq(fast_stats["per_query"], node_bytes, 48, 20, n, kms, l2_peak),
                         "limiter": "instruction issue and dependent L2 loads of an L2-resident tree; DRAM traffic "
                                    "is below the algorithmic bytes (ncu, profiles/)"},
            "quantised": quantised,
            "clocks": clocks, "accuracy": accuracy,
        }
        if not args.no_loss:
            result["distance_loss"] = distance_loss_bench(local)
        if not args.no_batch:
            result["batched_scenes"] = batched_scenes_bench(local)
        if world == 1 and not args.no_cpu_baseline:
            result["cpu_baseline"] = cpu_baseline(v, f, pts)
        if not args.no_suite:
            del gpu
            result["suite"] = suite_records(args, "c1,rays,c3,sil3d", cpu_budget=4.0)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(result), flush=True)


def run_reference(args):
    """The reference's own CPU implementation of the path: its Scene<3> built by its own
    SAH build and queried through its public bundled API (Scene::findClosestPoints over
    std::vector, one std::thread per hardware thread), compiled on this host from its
    headers (oracle/_ref). The scalar Bvh (the configuration's comparator) and the
    vectorised Mbvh (Enoki, FCPW_SIMD_WIDTH=4) are both measured on the warm-up calls;
    the faster one is timed on every step, all queries of the workload per step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from fcpw_gb300 import records as R
    from oracle import reference as REF
    base = {"impl": "reference", "metric": METRIC, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded torus + uniform queries)"}
    if not REF.available():
        print(json.dumps({"impl": "reference", "unavailable": "the reference's CPU headers are not staged on this "
                                                              "host (oracle/build.py), so it cannot be compiled"}))
        return
    v, f, pts = make_workload(0, args.queries)
    n = len(pts)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    refs = reference_cpu(3, v, f)
    build_s = time.perf_counter() - t0
    sph = R.make_spheres(pts, R.FLT_MAX)
    m = max(1, n // 16)
    warm = {}
    for name in ("scalar", "vectorized"):
        if refs.get(name) is None:
            continue
        secs = [refs[name].closest_points_timed(sph[:m])[1] for _ in range(max(1, args.warmup))]
        warm[name] = m / min(secs)
    best = max(warm, key=warm.get)
    # every step answers all n queries unless K such steps would take more than about 4 minutes
    budget_s = 240.0
    sample = n if args.steps * n / warm[best] <= budget_s else max(m, int(budget_s * warm[best] / args.steps))
    times = []
    for _ in range(args.steps):
        out, sec = refs[best].closest_points_timed(sph[:sample])
        times.append(sec)
    ms = 1e3 * sum(times) / len(times)
    value = sample / (ms / 1e3)
    builds = {best: {"queries_per_s": value, "queries_per_step": sample, "ms_per_step": ms}}
    other = [k for k in warm if k != best]
    if other:
        sec = refs[other[0]].closest_points_timed(sph[:sample])[1]
        builds[other[0]] = {"queries_per_s": sample / sec, "queries_per_step": sample, "ms_per_step": 1e3 * sec,
                            "note": "one call, for the record"}
    width = REF.simd_width() if "vectorized" in warm else 0
    if "vectorized" not in warm:
        from oracle.build import REF_SIMD_ERROR
        why = REF_SIMD_ERROR.read_text().strip().splitlines()[:1] if REF_SIMD_ERROR.exists() else []
        builds["vectorized"] = {"unavailable": "the reference's Enoki build (vectorize=true, FCPW_SIMD_WIDTH=4) "
                                               "does not compile on this host" + (f": {why[0]}" if why else "")}
    desc = (f"{sample:,} of the {n:,} queries per step through the reference's Scene<3>::findClosestPoints "
            f"({best}{f', Mbvh FCPW_SIMD_WIDTH={width}' if best == 'vectorized' else ', binary SAH Bvh'}), its own "
            f"std::thread split over {threads} hardware threads; timed inside the call")
    print(json.dumps({
        **base, "value": value, "ms_per_step": ms,
        "config": {"workload": "closest point, seeded torus 1,048,576 triangles, 4,194,304 queries "
                               "uniform in [-2,2]^3 per GPU, r2 = FLT_MAX, SAH BVH",
                   "queries_per_step": sample, "same_config": sample == n, "build": best,
                   "reference_build_s": round(build_s, 2), "builds": builds,
                   "host": {"machine": platform.machine(), "cpu": _cpu_model(), "threads": threads}},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "reference", "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# Arm CPU part numbers (the MIDR part field /proc/cpuinfo reports as "CPU part")
_ARM_PARTS = {"0xd40": "Neoverse-V1", "0xd49": "Neoverse-N2", "0xd4f": "Neoverse-V2 (Grace)", "0xd0c": "Neoverse-N1",
              "0xd8e": "Neoverse-N3", "0xd84": "Neoverse-V3"}


def _cpu_model() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            key = line.lower()
            if key.startswith(("model name", "hardware")):
                return line.split(":", 1)[1].strip()
            if key.startswith("cpu part"):
                part = line.split(":", 1)[1].strip().lower()
                return _ARM_PARTS.get(part, f"Arm CPU part {part}")
    except OSError:
        pass
    return platform.processor() or "unknown"


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.suite:
        run_suite(a)
    else:
        run_ours(a)
