#!/usr/bin/env python
"""Benchmark of the GPU BVH pipeline on one GB300: LBVH build -> Bittner13 optimizer -> closest hit.

Workload (the large single scene): 4,194,304 fp32 triangles (a 64-component Gaussian mixture plus a
724 x 724 two-triangle-per-cell ground grid, seeded), 63-bit Morton codes, LBVH (karras topology),
200 parallel Bittner13 iterations at 1%, then 1920 x 1080 primary rays plus one cosine-weighted
diffuse bounce per hit. Synthetic inputs stand in for the reference's mesh files.

One step = build + optimize + trace. `value` is the build + optimize time in ms (inputs already in
HBM); `e2e` is the same metric through the C ABI with the mesh copied from pinned host memory
and the optimised node array copied back inside the timed region. `batched` builds, optimises and
traces 256 meshes of uneven size as one captured graph after autotuning. `learned_vs_plain` trains the
learned reinsertion scorer (32 seeded 65,536-triangle scenes, about 52M logged pairs, 20k AdamW
steps) and times build + optimisation to equal SAH on an unseen scene, plain against learned.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload large|small]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "build+optimize ms at equal SAH (learned vs plain); Mrays/s closest-hit; HBM GB/s"
NODE_BYTES = 48


def workload(name: str):
    from bvhtest_gb300 import scenes
    if name == "large":
        vert, faces = scenes.large_scene()
        return dict(name="large", vert=vert, faces=faces, bits=63, topo="karras", iters=200,
                    camera=dict(pos=(5.0, 7.0, 5.0), lookAt=(5.0, 0.0, 5.0), up=(0.0, 0.0, 1.0), fov=60.0,
                                width=1920, height=1080),
                    desc=("large single scene: 4,194,304 triangles (64-component Gaussian mixture + 724x724 "
                          "ground grid), 63-bit Morton, karras LBVH, 200 Bittner13 iterations at 1% (32 chunks), "
                          "1920x1080 primary rays + 1 cosine-weighted bounce per hit"))
    if name == "stress":
        vert, faces = scenes.stress_scene()
        return dict(name="stress", vert=vert, faces=faces, bits=63, topo="karras", iters=300,
                    camera=dict(pos=(5.0, 16.0, 5.0), lookAt=(5.0, 0.0, 5.0), up=(0.0, 0.0, 1.0), fov=60.0,
                                width=1920, height=1080),
                    desc=("combined stress scene: 33,554,432 triangles (512 rotated boxes, 52x52 quads per face, "
                          "+ 256-component Gaussian mixture), 63-bit Morton, karras LBVH, 300 Bittner13 "
                          "iterations at 1%"))
    vert, faces = scenes.uniform_soup(65536, seed=1)
    return dict(name="small", vert=vert, faces=faces, bits=30, topo="refCompat", iters=100,
                camera=scenes.camera_default(),
                desc=("plain small scene: 65,536 triangles, 30-bit Morton, refCompat LBVH, 100 Bittner13 "
                      "iterations at 1%, 512x512 primary rays + 1 bounce"))


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_tflops():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        v = d.get("bf16_tflops")
        if v:
            return float(v), "measured"
    return 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (read-only queries)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(gpus: int):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x: float, world: int) -> float:
    """Maximum over ranks (the slowest replica sets the step time)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------------------------
# The reference's CPU path on the host cores (the oracle's restatement; see run_reference)
# ---------------------------------------------------------------------------------------------

# The SAH that "equal SAH" refers to: within 0.5% of the reference optimizer's SAH after its
# configured run (200 iterations of 32 chunks of 1%) from this scene's LBVH. The reference optimizer
# is Bittner13Par, the reference's CPU form of its chunked GPU optimizer (bittner13GPU itself is not
# deterministic): 108.68220964 is the SAH, summed in double, of the tree that the reference's own
# lib/builder/Bittner13Par.cpp produces (tests/golden/ref_pin.npz, key c2_par_sah, written by
# tests/golden/make_ref_golden.py from the reference's sources). Both arms run to the same number.
REF_SAH_200 = {"large": 108.68220964}
SAH_TARGET = {k: round(1.005 * v, 6) for k, v in REF_SAH_200.items()}
REF_BUDGET_S = 150.0  # wall-time budget of the reference arm's repeated steps


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def shared_config(w):
    """The workload as both arms describe it (no run-dependent values)."""
    n = int(w["faces"].shape[0])
    ref = REF_SAH_200.get(w["name"])
    return {"workload": w["desc"], "triangles": n, "nodes": 2 * n - 1, "sah_target": SAH_TARGET.get(w["name"]),
            "target": (f"within 0.5% of the reference optimizer's SAH after {w['iters']} Bittner13 iterations "
                       f"(32 chunks of 1%) from this scene's LBVH ({ref})" if ref else
                       f"{w['iters']} Bittner13 iterations (32 chunks of 1%)"),
            "parallelism": "single",
            "l2": "256 MB buffer written between GPU steps; inputs (201 MB) and nodes (403 MB) exceed L2"}


def reference_cpu_run(w, target):
    """One step of the reference's CPU path: the oracle's LBVH (the phases of LBVH_CUDA.cu on the
    host) and the oracle's Bittner13Par (byte-identical to lib/builder/Bittner13Par.cpp: heap
    search, first-come conflicts, nth_element + sort selection; 32 chunks of 1%), on all host
    threads, until the SAH reaches the target (at most the configured iteration count). The SAH
    evaluations that decide when to stop are not timed."""
    from oracle import pyoracle as orc
    t0 = time.perf_counter()
    nodes, _, _ = orc.lbvh_build(w["vert"], w["faces"], w["bits"], 1 if w["topo"] == "karras" else 0)
    build_ms = (time.perf_counter() - t0) * 1e3
    k, trace, iter_ms, st = orc.bittner_chunked_until(nodes, w["iters"], target, search_mode=1, heap_cap=16384,
                                                      conflict_rule=1, std_select=1)
    opt_ms = float(iter_ms.sum())
    return {"value": build_ms + opt_ms, "build_ms": build_ms, "optimize_ms": opt_ms, "iterations": k,
            "sah": float(trace[-1]), "reached": bool(trace[-1] <= target), "nodes": nodes,
            "skipped": st["skipped_conflict"] + st["skipped_invalid"], "items": st["items"]}


def reference_cpu_extras(w, nodes, rays_sample=65536, one_thread_iters=2):
    """Beside a full run: the same phases on one thread (LBVH + a few optimizer iterations, per
    iteration; not extrapolated into any headline), and the reference's stackless CPU tracer on a
    sample of the primary rays (all threads)."""
    from oracle import pyoracle as orc
    threads = orc.num_threads()
    orc.set_threads(1)
    try:
        t0 = time.perf_counter()
        one, _, _ = orc.lbvh_build(w["vert"], w["faces"], w["bits"], 1 if w["topo"] == "karras" else 0)
        b1 = (time.perf_counter() - t0) * 1e3
        k, _, ms, _ = orc.bittner_chunked_until(one, one_thread_iters, 0.0, search_mode=1, heap_cap=16384,
                                                conflict_rule=1, std_select=1)
    finally:
        orc.set_threads(threads)
    cam = w["camera"]
    org, dirs = orc.camera_rays(cam["pos"], cam["lookAt"], cam["up"], cam["fov"], cam["width"], cam["height"])
    sel = np.linspace(0, org.shape[0] - 1, rays_sample).astype(np.int64)
    t0 = time.perf_counter()
    orc.trace_cpu_reference(org[sel], dirs[sel], nodes, w["vert"], w["faces"])
    tr_s = time.perf_counter() - t0
    return {"one_thread": {"build_ms": round(b1, 1), "optimize_ms_per_iteration": round(float(ms.mean()), 1),
                           "iterations_timed": int(k)},
            "trace_mrays_per_s": round(rays_sample / tr_s / 1e6, 3), "trace_rays_sample": rays_sample}


def cpu_baseline_record(w, runs, extras):
    from oracle import pyoracle as orc
    r = runs[-1]
    v = statistics.mean(x["value"] for x in runs)
    return {"value": round(v, 1), "unit": "ms", "cores": orc.num_threads(), "kind": "port",
            "cpu_model": cpu_model(),
            "sample": (f"{len(runs)} full run(s) of the workload: the oracle's CPU LBVH + its Bittner13Par "
                       f"(byte-identical to the reference's) on {orc.num_threads()} threads to the target SAH, "
                       f"{r['iterations']} iterations"),
            "build_ms": round(statistics.mean(x["build_ms"] for x in runs), 1),
            "optimize_ms": round(statistics.mean(x["optimize_ms"] for x in runs), 1),
            "iterations": r["iterations"], "sah": round(r["sah"], 4), "reached_target": r["reached"],
            "skipped": r["skipped"], "items": r["items"], **extras}


def run_reference(args, w, rank, world):
    """--impl reference: the reference's CPU implementation of the path, timed on the host cores.

    The reference's own sources cannot run on the GPU machine (they are not there, and they need
    the math library its tree leaves empty), so its CPU path runs as the oracle's restatement,
    which tests/test_ref_pin.py pins byte for byte to the reference's compiled Bittner13Par. Each
    step is one full run of the workload to the same SAH as the GPU arm. A step takes tens of
    seconds, so the arm runs as many steps as fit in REF_BUDGET_S (at least one) and reports the
    steps it ran; there is no warm-up beyond the first step's page faults."""
    if rank != 0:
        return
    target = SAH_TARGET.get(w["name"], 0.0)
    runs = []
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        if runs:
            runs[-1].pop("nodes", None)  # keep only the last run's tree (400 MB each)
        runs.append(reference_cpu_run(w, target))
        step_s = time.perf_counter() - t0
        if len(runs) >= args.steps or (time.perf_counter() - t_start) + step_s > REF_BUDGET_S:
            break
    extras = reference_cpu_extras(w, runs[-1]["nodes"])
    cb = cpu_baseline_record(w, runs, extras)
    v = cb["value"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus,
            "steps": len(runs), "warmup": 0, "steps_requested": args.steps, "warmup_requested": args.warmup,
            "ms_per_step": v, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": shared_config(w), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------------------

def run_ours(args, w, rank, world, local):
    import torch
    from bvhtest_gb300 import api, native

    lib = native.load()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    vert_h, faces_h = w["vert"], w["faces"]
    n = int(faces_h.shape[0])
    n_nodes = 2 * n - 1
    vert = torch.from_numpy(vert_h).to(dev)
    faces = torch.from_numpy(faces_h.view(np.int32)).to(dev)
    nodes = api.empty_nodes(n_nodes)
    lbvh = api.LBVH(n, w["bits"], w["topo"])
    lbvh.build(vert, faces, nodes)
    torch.cuda.synchronize()
    opt = api.Bittner13GPU(nodes, num_nodes=n_nodes, profile=not args.no_kernel_events)
    tracer = api.Tracer(n_nodes)
    cam = w["camera"]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def ev():
        e = torch.cuda.Event(enable_timing=True)
        e.record(stream)
        return e

    # The primary rays' traversal schedule, chosen by timing both on this tree (the reference's
    # rayBundles option): one ray per thread, or a warp of neighbouring rays as one bundle.
    tracer.update(nodes, num_nodes=n_nodes)
    sched = {}
    for bundles in (False, True):
        for _ in range(2):
            tracer.trace_image(vert, faces, cam, ray_bundles=bundles)
        e0 = ev()
        for _ in range(5):
            tracer.trace_image(vert, faces, cam, ray_bundles=bundles)
        e1 = ev()
        torch.cuda.synchronize()
        sched["bundle_ms" if bundles else "per_ray_ms"] = round(e0.elapsed_time(e1) / 5, 4)
    use_bundles = sched["bundle_ms"] < sched["per_ray_ms"]
    sched["chosen"] = "bundle" if use_bundles else "per_ray"

    def step():
        marks = [ev()]
        lbvh.init_tri_data(vert, faces)
        marks.append(ev())
        lbvh.calc_morton(vert, faces)
        marks.append(ev())
        lbvh.sort(n)
        marks.append(ev())
        lbvh.build_tree(vert, faces, nodes)
        marks.append(ev())
        opt.run(w["iters"])
        marks.append(ev())
        tracer.update(nodes, num_nodes=n_nodes)  # traversal records of this tree, timed with the trace
        img, hits = tracer.trace_image(vert, faces, cam, ray_bundles=use_bundles)
        bounce, _, _ = tracer.trace_bounce(vert, faces, cam, hits, seed=17)
        marks.append(ev())
        return marks, hits, bounce

    launches0 = lib.bvhgb_launch_count()
    for _ in range(args.warmup):
        flush.fill_(1)
        step()
    torch.cuda.synchronize()
    st0 = opt.stats()
    phases = {"bounds": [], "morton": [], "sort": [], "topology_refit": [], "optimize": [], "trace": []}
    step_ms, hits_n = [], []
    c0 = lib.bvhgb_launch_count()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            barrier(world)
            marks, hits, bounce = step()
            torch.cuda.synchronize()
            t = [marks[i].elapsed_time(marks[i + 1]) for i in range(len(marks) - 1)]
            for k, v in zip(phases, t):
                phases[k].append(v)
            step_ms.append(marks[0].elapsed_time(marks[-1]))
            h = api.hits_to_numpy(hits)
            b = api.hits_to_numpy(bounce)
            hits_n.append((h.shape[0], int((h["prim"] != 0xFFFFFFFF).sum()), int((b["prim"] != 0xFFFFFFFF).sum())))
    c1 = lib.bvhgb_launch_count()
    st1 = opt.stats()
    search_ms, search_launches = opt.search_time() if not args.no_kernel_events else (0.0, 0)
    sah = api.calc_sah(nodes, 0, n_nodes)
    mean = {k: statistics.mean(v) for k, v in phases.items()}
    build_ms = mean["bounds"] + mean["morton"] + mean["sort"] + mean["topology_refit"]
    value = allmax(build_ms + mean["optimize"], world)
    ms_step = allmax(statistics.mean(step_ms), world)
    rays = hits_n[-1][0] + hits_n[-1][1]  # primary rays + one bounce per primary hit
    mrays = rays / (mean["trace"] * 1e-3) / 1e6
    gpu_launches = int((c1 - c0) / args.steps)  # graph replays count the kernels they hold

    # Build-phase algorithmic bytes (key bytes K, value bytes V = 4, P 8-bit digit passes), as the
    # scope's measurement section defines them for the reference's phases: scene reduce + Morton
    # 2 (12 + 36) N + (K + V) N; sort K N + P 2 (K + V) N; topology K N + 48 (2N - 1); refit
    # 2 * 48 (N - 1) + 48 (N - 1) + 48 N + 8 (N - 1). The fused build kernel moves less than the
    # separate topology + refit passes counted here.
    K = 8 if w["bits"] == 63 else 4
    P = (w["bits"] + 7) // 8
    alg = {"bounds": 48 * n, "morton": 48 * n + (K + 4) * n, "sort": K * n + P * 2 * (K + 4) * n,
           "topology_refit": K * n + NODE_BYTES * n_nodes + 2 * 48 * (n - 1) + 48 * (n - 1) + 48 * n + 8 * (n - 1)}
    peak, peak_kind = measured_peaks()
    build_bytes = sum(alg.values())
    build_gbs = build_bytes / (build_ms * 1e-3) / 1e9
    # Dominant kernel: the reinsertion search (bn13 patch), timed with CUDA events in the graph.
    visits = st1["nodesVisited"] - st0["nodesVisited"]
    launches_search = args.steps * w["iters"] * max(1, search_launches)
    per_launch_bytes = visits * NODE_BYTES / launches_search
    per_launch_ms = search_ms / max(1, search_launches)
    ach = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9 if per_launch_ms > 0 else 0.0
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get(w["name"], {}).get("bn13_patch")
    clocks = clk.summary()
    if rank != 0:
        return
    if args.no_cpu_baseline:
        cpu_rec = {"value": None, "unit": "ms", "cores": 0, "kind": "port", "sample": "skipped"}
    else:
        cpu_runs = [reference_cpu_run(w, SAH_TARGET.get(w["name"], 0.0))]
        cpu_rec = cpu_baseline_record(w, cpu_runs, reference_cpu_extras(w, cpu_runs[-1]["nodes"]))
        del cpu_runs

    # e2e through the C ABI: pinned host mesh -> device, build, optimize, node array -> pinned host.
    vh = torch.from_numpy(vert_h).pin_memory()
    fh = torch.from_numpy(faces_h.view(np.int32)).pin_memory()
    nh = torch.empty((n_nodes, 12), dtype=torch.int32).pin_memory()
    vd = torch.empty_like(vert)
    fd = torch.empty_like(faces)
    e2e = []
    for i in range(args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0 = ev()
        vd.copy_(vh, non_blocking=True)
        fd.copy_(fh, non_blocking=True)
        lbvh.build(vd, fd, nodes)
        opt.run(w["iters"])
        nh.copy_(nodes[:n_nodes], non_blocking=True)
        e1 = ev()
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e.append(e0.elapsed_time(e1))
    e2e_ms = statistics.mean(e2e)

    plain = {"iterations": w["iters"], "build_optimize_ms": round(value, 3), "e2e_ms": round(e2e_ms, 3),
             "optimize_ms_per_iteration": round(mean["optimize"] / w["iters"], 4), "sah": round(sah, 4),
             "gpu_launches": gpu_launches, "clocks": clocks}
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(value, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": shared_config(w),
        "iterations": w["iters"], "method": "plain (inefficiency) selection, the configured iteration count",
        "batch_per_iteration": opt.batch_size,
        "step": "one pass of the hot path = LBVH build + optimisation to the target SAH; the trace is timed apart",
        "build_ms": round(build_ms, 3), "optimize_ms": round(mean["optimize"], 3),
        "optimize_ms_per_iteration": round(mean["optimize"] / w["iters"], 4),
        "trace_ms": round(mean["trace"], 3), "mrays_per_s": round(mrays, 1), "rays_per_step": rays,
        "primary_schedule": sched,
        "build_phase_ms": {k: round(mean[k], 4) for k in alg},
        "build_hbm_gbs": round(build_gbs, 1),
        "build_roofline": {"bound": "hbm", "achieved": round(build_gbs, 1), "peak": peak, "unit": "GB/s",
                           "frac": round(build_gbs / peak, 4), "peak_kind": peak_kind,
                           "bytes_per_triangle": round(build_bytes / n, 1)},
        "sah": round(sah, 4),
        "bittner": {"applied": st1["applied"] - st0["applied"], "items": st1["items"] - st0["items"],
                    "skipped_conflict": st1["skippedConflict"] - st0["skippedConflict"],
                    "heap_overflow": st1["heapOverflow"] - st0["heapOverflow"]},
        "roofline": {"kernel": "bn13 patch (reinsertion search)", "bound": "hbm", "achieved": round(ach, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 5), "traffic": traffic,
                     "peak_kind": peak_kind, "ms_per_launch": round(per_launch_ms, 4),
                     "algorithmic_bytes_per_launch": int(per_launch_bytes)},
        "cpu_baseline": cpu_rec,
        "e2e": {"value": round(e2e_ms, 3), "unit": "ms", "h2d_bytes_per_step": int(vert_h.nbytes + faces_h.nbytes),
                "d2h_bytes_per_step": int(n_nodes * NODE_BYTES)},
        "gpu_launches": gpu_launches,
        "clocks": clocks,
        "plain": plain,
    }
    scorer = None
    if not args.no_learned or not args.no_stress:
        from bvhtest_gb300 import learned
        scorer, train = learned.train_family("large")
    if not args.no_learned:
        ref200 = REF_SAH_200.get(w["name"], sah)
        line["plain_sah_vs_reference"] = {"gpu_plain_sah": round(sah, 6), "reference_sah": ref200,
                                          "relative": round(sah / ref200 - 1.0, 6), "iterations": w["iters"]}
        big = learned_large(args, w, dev, flush, stream, vert, faces, nodes, lbvh, SAH_TARGET.get(w["name"], sah), lib,
                            ev, vh,
                            fh, nh, vd, fd,
                            per_launch_ms * max(1, search_launches), scorer, train)
        line["learned"] = big
        if "build_optimize_ms" in big:
            # the headline: build + optimisation to the SAH of the configured plain run (equal SAH)
            line["value"] = big["build_optimize_ms"]
            line["e2e"]["value"] = big["e2e_ms"]
            line["gpu_launches"] = big["gpu_launches"]
            line["clocks"] = big["clocks"]
            line["sah"] = big["sah"]
            line["method"] = big["method"]
            line["iterations"] = big["iterations"]
            line["optimize_ms"] = big["optimize_ms"]
            line["optimize_ms_per_iteration"] = round(big["optimize_ms"] / big["iterations"], 4)
            line["ms_per_step"] = big["build_optimize_ms"]
            if big.get("roofline"):
                line["roofline_plain"] = line["roofline"]  # the plain arm's search, for comparison
                line["roofline"] = big["roofline"]
        line["learned_vs_plain"] = learned_arm(args, dev, flush, stream)
    if not args.no_batch:
        line["batched"] = batch_arm(args, dev, flush)
    if not args.no_stress:
        line["stress"] = stress_arm(args, dev, flush, scorer)
    print(json.dumps(line), flush=True)


def stress_arm(args, dev, flush, scorer):
    """Combined stress test: 33,554,432 triangles (512 randomly rotated boxes, 52 x 52 quads per face,
    and a 256-component Gaussian mixture), 63-bit Morton, karras LBVH; 300 plain Bittner13
    iterations set the target, the learned policy (scorer of the large-scene family, alternating with
    the plain measure) runs until its SAH is within 0.5% of it; then 16,777,216 incoherent rays in 16
    batches of 64k to 4M (origins uniform in the scene box, directions uniform on the sphere,
    tmax = inf). The plain run is timed once (per-iteration events, no host synchronisation), the
    learned run W + K times."""
    import torch
    from bvhtest_gb300 import api, native, scenes

    lib = native.load()
    vert_h, faces_h = scenes.stress_scene()
    n = int(faces_h.shape[0])
    n_nodes = 2 * n - 1
    v = torch.from_numpy(vert_h).to(dev)
    f = torch.from_numpy(faces_h.view(np.int32)).to(dev)
    nodes = api.empty_nodes(n_nodes)
    lbvh = api.LBVH(n, 63, "karras")
    rebuild = lambda: lbvh.build(v, f, nodes)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    plain_iters = 300

    def events_run(opt, iters, first=0):
        flush.fill_(1)
        torch.cuda.synchronize()
        marks = [ev()]
        marks[0].record()
        rebuild()
        m = ev()
        m.record()
        marks.append(m)
        opt.iteration = first
        for _ in range(iters):
            opt.run(1)
            m = ev()
            m.record()
            marks.append(m)
        torch.cuda.synchronize()
        return [marks[0].elapsed_time(x) for x in marks[1:]]  # build, then after each iteration

    # warm-up of every kernel, then the untimed calibration: the SAH after each plain iteration
    rebuild()
    popt = api.Bittner13GPU(nodes, num_nodes=n_nodes)
    popt.run(3)
    rebuild()
    popt.iteration = 0
    trace = []
    for _ in range(plain_iters):
        popt.run(1)
        trace.append(api.calc_sah(nodes))
    target = 1.005 * trace[-1]
    kp = next(i + 1 for i, x in enumerate(trace) if x <= target)
    pt = events_run(popt, plain_iters)
    plain_sah = api.calc_sah(nodes)
    pst = popt.stats()
    popt.close()
    # learned selection until the target: the default policy (scorer first, alternating with plain)
    # and the same alternation started with a plain iteration (iteration counter at 1)
    lopt = api.Bittner13GPU(rebuild(), num_nodes=n_nodes)
    lopt.set_scorer(scorer, 2)

    def first_hit(first):
        rebuild()
        lopt.iteration = first
        for it in range(1, plain_iters + 1):
            lopt.run(1)
            if api.calc_sah(nodes) <= target:
                return it
        return None
    k = first_hit(0)
    kf = first_hit(1)
    out = {
        "workload": ("33,554,432 triangles: 512 randomly rotated boxes (centres uniform in [0,10]^3, half extents "
                     "uniform in [0.1,0.6]) with 52 x 52 quads per face (16,613,376 triangles) and a 256-component "
                     "Gaussian mixture (16,941,056); 63-bit Morton, karras LBVH; learned Bittner13 until within 0.5% "
                     "of the SAH of 300 plain iterations; 16,777,216 incoherent rays in 16 batches of 64k..4M"),
        "triangles": n, "nodes": n_nodes,
        "build_ms": round(pt[0], 3),
        "build_hbm_gbs": round(n * 612.0 / (pt[0] * 1e-3) / 1e9, 1),
        "plain": {"iterations": plain_iters, "build_optimize_ms": round(pt[-1], 3), "sah": round(plain_sah, 4),
                  "sah_trace_300": round(trace[-1], 4), "first_within_0.5pct_iterations": kp,
                  "first_within_0.5pct_build_optimize_ms": round(pt[kp], 3),
                  "applied": pst["applied"], "skipped_conflict": pst["skippedConflict"]},
        "sah_target": round(target, 4),
    }
    if k is None:
        out["error"] = "learned selection did not come within 0.5% of the plain SAH in 300 iterations"
    else:
        times = []
        c0 = lib.bvhgb_launch_count()
        for i in range(1 + args.steps):
            if i == 1:
                c0 = lib.bvhgb_launch_count()
            t = events_run(lopt, k)
            if i >= 1:
                times.append(t)
        launches = (lib.bvhgb_launch_count() - c0) // args.steps
        lb = statistics.mean(t[0] for t in times)
        lt = statistics.mean(t[-1] for t in times)
        out["learned"] = {"iterations": k, "build_optimize_ms": round(lt, 3), "build_ms": round(lb, 3),
                          "sah": round(api.calc_sah(nodes), 4), "gpu_launches": int(launches),
                          "policy": "scorer iterations alternating with plain ones (plainEvery 2)"}
        out["wall_time_ratio_vs_plain_300"] = round(lt / pt[-1], 4)
        out["wall_time_ratio_vs_plain_first_within_0.5pct"] = round(lt / pt[kp], 4)
    if kf is not None:
        times = [events_run(lopt, kf, first=1) for _ in range(1 + args.steps)][1:]
        lt = statistics.mean(t[-1] for t in times)
        out["learned_plain_first"] = {
            "iterations": kf, "build_optimize_ms": round(lt, 3), "sah": round(api.calc_sah(nodes), 4),
            "policy": "the same alternation started with a plain iteration (on this scene the first plain "
                      "iteration gains most for the least time)",
            "wall_time_ratio_vs_plain_first_within_0.5pct": round(lt / pt[kp], 4)}
    lopt.close()
    # incoherent rays in 16 batches through the optimised tree
    lo, hi = vert_h.min(0), vert_h.max(0)
    del vert_h, faces_h
    org_h, dir_h, sizes = scenes.stress_rays(lo, hi)
    org = torch.from_numpy(org_h).to(dev)
    dirs = torch.from_numpy(dir_h).to(dev)
    tracer = api.Tracer(n_nodes)
    tracer.update(nodes, num_nodes=n_nodes).trace_rays(v, f, org[:65536], dirs[:65536])  # warm-up
    flush.fill_(1)
    torch.cuda.synchronize()
    marks = [ev()]
    marks[0].record()
    tracer.update(nodes, num_nodes=n_nodes)  # the traversal records, timed with the first batch
    hits, off = [], 0
    for sz in sizes:
        hits.append(tracer.trace_rays(v, f, org[off:off + sz], dirs[off:off + sz]))
        off += sz
        m = ev()
        m.record()
        marks.append(m)
    torch.cuda.synchronize()
    per = [marks[i].elapsed_time(marks[i + 1]) for i in range(len(sizes))]
    total = sum(per)
    h = api.hits_to_numpy(torch.cat(hits))
    out["trace"] = {"rays": int(sum(sizes)), "batches": list(sizes), "ms": round(total, 3),
                    "mrays_per_s": round(sum(sizes) / (total * 1e-3) / 1e6, 1),
                    "batch_mrays_per_s": [round(sz / (t * 1e-3) / 1e6, 1) for sz, t in zip(sizes, per)],
                    "hit_fraction": round(float((h["prim"] != 0xFFFFFFFF).mean()), 4),
                    "errors": api.trace_errors()}
    out["lbvh_errors"] = lbvh.errors()
    lbvh.close()
    return out


def batch_arm(args, dev, flush):
    """Batched build (256 meshes, log-uniform 1,024..524,288 triangles, about 20M in total): autotune,
    then time the whole pipeline (LBVH, 50 Bittner13 iterations, 65,536 random rays per mesh) as one
    captured CUDA graph, plus each phase on its own."""
    import torch
    from bvhtest_gb300 import api, native, scenes

    lib = native.load()
    iters, rays = 50, 65536
    vert_h, faces_h, counts = scenes.batch_meshes(256, 1024, 524288, seed=9)
    v = torch.from_numpy(vert_h).to(dev)
    f = torch.from_numpy(faces_h.view(np.int32)).to(dev)
    b = api.Batch(counts)
    nodes = b.empty_nodes()
    hits = torch.empty(256 * rays, dtype=torch.int64, device=dev)
    tune = b.autotune(v, f, nodes, rays, hits, seed=11)

    def timed(fn):
        out = []
        for i in range(args.warmup + args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            if i >= args.warmup:
                out.append(e0.elapsed_time(e1))
        return statistics.mean(out)

    c0 = lib.bvhgb_launch_count()
    graph_ms = timed(lambda: b.run(v, f, nodes, iters, rays, hits, seed=11))
    launches = (lib.bvhgb_launch_count() - c0) // (args.warmup + args.steps)
    build_ms = timed(lambda: b.build(v, f, nodes))

    def build_opt():
        b.build(v, f, nodes)
        b.optimize(nodes, iters)
    opt_ms = timed(build_opt) - build_ms
    trace_ms = timed(lambda: b.trace_random(nodes, v, f, rays, seed=11))
    st, err = b.stats()
    h = api.hits_to_numpy(hits)
    n = int(counts.sum())
    return {
        "workload": ("256 meshes, triangle counts log-uniform in [1,024, 524,288], each a Gaussian mixture in the "
                     "unit cube with 1-16 clusters and its own seed; 30-bit Morton, refCompat LBVH, 50 Bittner13 "
                     "iterations at 1% (32 chunks), 65,536 random rays per mesh (origins in the mesh box grown "
                     "1.5x, directions uniform on the sphere)"),
        "meshes": 256, "triangles": n, "min_triangles": int(counts.min()), "max_triangles": int(counts.max()),
        "pipeline_ms": round(graph_ms, 3), "build_ms": round(build_ms, 3), "optimize_ms": round(opt_ms, 3),
        "trace_ms": round(trace_ms, 3), "rays": 256 * rays, "mrays_per_s": round(256 * rays / (trace_ms * 1e-3) / 1e6, 1),
        "build_mtris_per_s": round(n / (build_ms * 1e-3) / 1e6, 1), "gpu_launches": int(launches),
        "hit_fraction": round(float((h["prim"] != 0xFFFFFFFF).mean()), 4), "errors": err,
        "autotune": tune, "launch": "one CUDA graph per pipeline (build + iterations + trace)",
    }


def first_hit(opt, nodes, target, max_iters, rebuild):
    """Untimed calibration: iterations until the SAH first drops to <= target (None if never)."""
    from bvhtest_gb300 import api
    rebuild()
    opt.iteration = 0
    for it in range(1, max_iters + 1):
        opt.step()
        if api.calc_sah(nodes) <= target:
            return it
    return None


def learned_large(args, w, dev, flush, stream, vert, faces, nodes, lbvh, target, lib, ev, vh, fh, nh, vd, fd,
                  search_ms_per_iteration, scorer, train):
    """Learned selection (alternating with the plain measure) on the benchmark scene until the SAH of
    the configured plain run is reached; the plain optimizer's first hit of the same SAH beside it."""
    import torch
    from bvhtest_gb300 import api

    n = int(w["faces"].shape[0])
    n_nodes = 2 * n - 1
    rebuild = lambda: lbvh.build(vert, faces, nodes)
    lopt = api.Bittner13GPU(rebuild(), num_nodes=n_nodes)
    lopt.set_scorer(scorer, 2)
    k = first_hit(lopt, nodes, target, w["iters"], rebuild)
    popt = api.Bittner13GPU(rebuild(), num_nodes=n_nodes)
    kp = first_hit(popt, nodes, target, w["iters"], rebuild)
    out = {"train": train, "sah_target": round(target, 4), "plain_first_hit_iterations": kp}
    if k is None:
        out["error"] = "learned selection did not reach the plain SAH within the configured iterations"
        return out

    def timed(opt, iters, with_clocks=False):
        res, c0 = [], lib.bvhgb_launch_count()
        sampler = ClockSampler(torch.cuda.current_device()) if with_clocks else None
        if sampler:
            sampler.__enter__()
        for i in range(args.warmup + args.steps):
            if i == args.warmup:
                c0 = lib.bvhgb_launch_count()
            flush.fill_(1)
            torch.cuda.synchronize()
            e0 = ev()
            rebuild()
            e1 = ev()
            opt.iteration = 0
            opt.run(iters)
            e2 = ev()
            torch.cuda.synchronize()
            if i >= args.warmup:
                res.append((e0.elapsed_time(e1), e1.elapsed_time(e2)))
        c1 = lib.bvhgb_launch_count()
        if sampler:
            sampler.__exit__(None, None, None)
        b = statistics.mean(r[0] for r in res)
        o = statistics.mean(r[1] for r in res)
        return b, o, int((c1 - c0) / args.steps), (sampler.summary() if sampler else None)

    lb, lo_, l_launch, l_clocks = timed(lopt, k, with_clocks=True)
    l_sah = api.calc_sah(nodes)
    pb, po_, _, _ = timed(popt, kp if kp else w["iters"])
    # e2e through the C ABI with host buffers
    e2e = []
    for i in range(args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0 = ev()
        vd.copy_(vh, non_blocking=True)
        fd.copy_(fh, non_blocking=True)
        lbvh.build(vd, fd, nodes)
        lopt.iteration = 0
        lopt.run(k)
        nh.copy_(nodes[:n_nodes], non_blocking=True)
        e1 = ev()
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e.append(e0.elapsed_time(e1))
    # The reinsertion search of the learned run, timed with kernel events in an untimed pass (that
    # workspace records events around every search launch; the timed runs above have none).
    prof = api.Bittner13GPU(rebuild(), num_nodes=n_nodes, profile=True)
    prof.set_scorer(scorer, 2)
    for _ in range(2):  # warm-up: both iteration graphs captured
        rebuild()
        prof.iteration = 0
        prof.run(k)
    rebuild()
    prof.iteration = 0
    visits0 = prof.stats()["nodesVisited"]
    s_ms, s_launches = 0.0, 0
    for _ in range(k):
        prof.run(1)
        torch.cuda.synchronize()
        ms_i, n_i = prof.search_time()
        s_ms += ms_i
        s_launches += n_i
    s_visits = prof.stats()["nodesVisited"] - visits0
    prof.close()
    search_roof = None
    if s_launches and s_ms > 0:
        peak, peak_kind = measured_peaks()
        bpl = s_visits * NODE_BYTES / s_launches
        mpl = s_ms / s_launches
        ach_s = bpl / (mpl * 1e-3) / 1e9
        tfile = ROOT / "profiles" / "traffic.json"
        traffic_l = (json.loads(tfile.read_text()).get(w["name"], {}).get("bn13_patch_learned")
                     if tfile.exists() else None)
        search_roof = {"kernel": "bn13 patch (reinsertion search), learned run", "bound": "hbm",
                       "achieved": round(ach_s, 1), "peak": peak, "unit": "GB/s", "frac": round(ach_s / peak, 5),
                       "traffic": traffic_l, "peak_kind": peak_kind, "ms_per_launch": round(mpl, 4),
                       "algorithmic_bytes_per_launch": int(bpl), "launches": int(s_launches)}
    # the scorer's inference kernel, timed alone on this scene's feature rows
    inner = lopt.inner_nodes()
    x = api.LrFeatures(n_nodes)(nodes, inner)
    for _ in range(3):
        scorer.forward(x)
    torch.cuda.synchronize()
    e0 = ev()
    reps = 10
    for _ in range(reps):
        scorer.forward(x)
    e1 = ev()
    torch.cuda.synchronize()
    mlp_ms = e0.elapsed_time(e1) / reps
    flops = 2.0 * (24 * 64 + 64 * 64 + 64) * inner.shape[0]
    tf_peak, tf_kind = measured_tflops()
    learned_iters = (k + 1) // 2
    roof = search_roof  # the dominant kernel of the learned run: the search, unless the scorer outweighs it
    if mlp_ms * learned_iters >= (s_ms if s_launches else search_ms_per_iteration * k):
        ach = flops / (mlp_ms * 1e-3) / 1e12
        roof = {"kernel": "scorer MLP forward (24-64-64-1, BF16 in, FP32 accumulate)", "bound": "tensor",
                "achieved": round(ach, 2), "peak": tf_peak, "unit": "TFLOP/s", "frac": round(ach / tf_peak, 5),
                "peak_kind": tf_kind, "traffic": None, "ms_per_launch": round(mlp_ms, 4),
                "algorithmic_flops_per_launch": int(flops)}
    return {
        "method": ("learned selection alternating with the plain measure (plainEvery 2) until the SAH is "
                   f"within 0.5% of the reference optimizer's after {w['iters']} iterations; scorer trained in "
                   "this run on 8 seeded 262,144-triangle scenes of the same generator (the benchmark scene is "
                   "not among them)"),
        "iterations": k, "learned_iterations": learned_iters, "plain_iterations": k - learned_iters,
        "build_optimize_ms": round(lb + lo_, 3), "build_ms": round(lb, 3), "optimize_ms": round(lo_, 3),
        "e2e_ms": round(statistics.mean(e2e), 3), "sah": round(l_sah, 4), "sah_target": round(target, 4),
        "gpu_launches": l_launch, "clocks": l_clocks,
        "build_optimize_ms_with_training": round(lb + lo_ + 1e3 * (train.get("log_s", 0.0) + train.get("train_s", 0.0)),
                                                 1),
        "plain_first_hit_iterations": kp, "plain_first_hit_build_optimize_ms": round(pb + po_, 3),
        "wall_time_ratio_vs_plain_first_hit": round((lb + lo_) / (pb + po_), 4),
        "mlp_forward_ms": round(mlp_ms, 4), "mlp_rows": int(inner.shape[0]),
        "roofline": roof, "train": train,
    }


# ---------------------------------------------------------------------------------------------
# Learned scorer against the plain measure (uniform 65,536-triangle scenes)
# ---------------------------------------------------------------------------------------------

LEARNED_N, LEARNED_SCENES, LEARNED_ITERS, LEARNED_EVERY, LEARNED_STEPS = 65536, 32, 100, 4, 20000


def learned_arm(args, dev, flush, stream):
    """Train the scorer on pairs logged from plain runs over 32 seeded scenes, then time LBVH build +
    optimisation to the plain optimizer's 100-iteration SAH on an unseen scene, plain vs learned."""
    import torch
    from bvhtest_gb300 import api, learned, scenes

    n = LEARNED_N
    scorer, train = learned.train_family("uniform", steps=LEARNED_STEPS)

    vert_h, faces_h = scenes.uniform_soup(n, seed=1)  # the training scenes use seeds 1000..1031
    vert = torch.from_numpy(vert_h).to(dev)
    faces = torch.from_numpy(faces_h.view(np.int32)).to(dev)
    nodes = api.empty_nodes(2 * n - 1)
    lbvh = api.LBVH(n, 30, "refCompat")
    plain = api.Bittner13GPU(lbvh.build(vert, faces, nodes))
    sah0 = api.calc_sah(nodes)
    plain.run(LEARNED_ITERS)
    target = api.calc_sah(nodes)
    lrn = api.Bittner13GPU(lbvh.build(vert, faces, nodes))
    lrn.set_scorer(scorer, 2)
    k_learned = None
    for it in range(1, LEARNED_ITERS + 1):  # calibration (untimed): iterations to reach the target
        lrn.step()
        if api.calc_sah(nodes) <= target:
            k_learned = it
            break
    if k_learned is None:
        return {"workload": "uniform 65,536 triangles", "error": "learned selection did not reach the plain SAH"}

    def timed(opt, iters):
        out = []
        for i in range(args.warmup + args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lbvh.build(vert, faces, nodes)
            opt.iteration = 0
            opt.run(iters)
            e1.record(stream)
            torch.cuda.synchronize()
            if i >= args.warmup:
                out.append(e0.elapsed_time(e1))
        return statistics.mean(out), api.calc_sah(nodes)

    k_plain = None  # plain first reaches its own 100-iteration SAH before iteration 100 and hovers
    lbvh.build(vert, faces, nodes)
    plain.iteration = 0
    for it in range(1, LEARNED_ITERS + 1):
        plain.step()
        if api.calc_sah(nodes) <= target:
            k_plain = it
            break
    plain_ms, plain_sah = timed(plain, LEARNED_ITERS)
    first_ms, _ = timed(plain, k_plain)
    learned_ms, learned_sah = timed(lrn, k_learned)
    lbvh.build(vert, faces, nodes)
    lrn.iteration = 0
    lrn.run(LEARNED_ITERS)
    sah_learned_full = api.calc_sah(nodes)
    return {
        "workload": ("uniform 65,536 triangles (seed 1, unseen in training), 30-bit Morton, refCompat LBVH; "
                     "target = SAH after 100 plain Bittner13 iterations at 1%"),
        "sah_start": round(sah0, 4), "sah_target": round(target, 4),
        "plain": {"iterations": LEARNED_ITERS, "build_optimize_ms": round(plain_ms, 3), "sah": round(plain_sah, 4),
                  "first_hit_iterations": k_plain, "first_hit_build_optimize_ms": round(first_ms, 3)},
        "learned": {"iterations": k_learned, "build_optimize_ms": round(learned_ms, 3), "sah": round(learned_sah, 4),
                    "sah_after_100": round(sah_learned_full, 4),
                    "policy": "scorer iterations alternating with plain ones (plainEvery 2)"},
        "wall_time_ratio": round(learned_ms / first_ms, 4),
        "wall_time_ratio_vs_100_plain": round(learned_ms / plain_ms, 4),
        "train": train,
    }


def run_batch_phase(args):
    """--only batch: the batched 256-mesh scene, build + args.iters Bittner13 iterations per run."""
    import torch
    from bvhtest_gb300 import api, scenes
    vert_h, faces_h, counts = scenes.batch_meshes(256, 1024, 524288, seed=9)
    v = torch.from_numpy(vert_h).cuda()
    f = torch.from_numpy(faces_h.view(np.int32)).cuda()
    b = api.Batch(counts, topology=args.batch_topology)
    nodes = b.empty_nodes()
    iters = args.iters if args.iters is not None else 50
    times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.build(v, f, nodes)
        b.optimize(nodes, iters)
        e1.record()
        torch.cuda.synchronize()
        if i >= args.warmup:
            times.append(e0.elapsed_time(e1))
    st, err = b.stats()
    print(f"batch: {statistics.mean(times):.3f} ms mean over {args.steps} runs ({iters} iterations, "
          f"{args.batch_topology}); visits {st['nodesVisited']} items {st['items']} applied {st['applied']} err {err}",
          flush=True)


def run_phase(args, w):
    """--only PHASE: repeat one phase of the pipeline (for profilers; prints one timing line, not the
    benchmark record)."""
    import torch
    from bvhtest_gb300 import api
    if args.only == "batch":
        return run_batch_phase(args)
    if args.only == "stress":
        import torch
        from bvhtest_gb300 import api, learned
        scorer = api.Mlp.load(args.scorer) if args.scorer else learned.train_family("large")[0]
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        print(json.dumps(stress_arm(args, torch.device("cuda"), flush, scorer)), flush=True)
        return
    n = int(w["faces"].shape[0])
    vert = torch.from_numpy(w["vert"]).cuda()
    faces = torch.from_numpy(w["faces"].view(np.int32)).cuda()
    nodes = api.empty_nodes(2 * n - 1)
    lbvh = api.LBVH(n, w["bits"], w["topo"])
    lbvh.build(vert, faces, nodes)
    opt = api.Bittner13GPU(nodes, num_nodes=2 * n - 1) if args.only == "optimize" else None
    tracer = api.Tracer(2 * n - 1) if args.only == "trace" else None
    if opt is not None and args.scorer:
        scorer = api.Mlp.load(args.scorer)
        opt.set_scorer(scorer, args.plain_every)
    times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        if args.only == "build":
            lbvh.build(vert, faces, nodes)
        elif args.only == "optimize":
            lbvh.build(vert, faces, nodes)
            opt.iteration = 0
            opt.run(w["iters"])
        else:
            tracer.update(nodes, num_nodes=2 * n - 1)
            img, hits = tracer.trace_image(vert, faces, w["camera"])
            tracer.trace_bounce(vert, faces, w["camera"], hits, seed=17)
        e1.record()
        torch.cuda.synchronize()
        if i >= args.warmup:
            times.append(e0.elapsed_time(e1))
    print(f"{args.only}: {statistics.mean(times):.4f} ms mean over {args.steps} runs ({w['name']})", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["large", "small", "stress"], default="large",
                    help="the benchmark scene (large); small and stress serve the --only profiling runs")
    ap.add_argument("--iters", type=int, default=None,
                    help="override the Bittner13 iteration count (profiling runs only; the headline uses the default)")
    ap.add_argument("--no-kernel-events", action="store_true",
                    help="do not bracket the search kernel with CUDA events (for runs under ncu)")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-scorer comparison")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched multi-mesh build")
    ap.add_argument("--no-stress", action="store_true", help="skip the 33.5M-triangle combined stress test")
    ap.add_argument("--batch-topology", choices=["refCompat", "karras"], default="refCompat",
                    help="with --only batch: the LBVH topology of the batched meshes")
    ap.add_argument("--only", choices=["build", "optimize", "trace", "batch", "stress"], default=None,
                    help="repeat one phase only and print its time (profiling runs; no benchmark record)")
    ap.add_argument("--scorer", default=None,
                    help="with --only optimize / stress: learned selection with these weights")
    ap.add_argument("--plain-every", type=int, default=2, help="with --scorer: every k-th iteration is plain")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_setup(args.gpus)
    w = workload(args.workload)
    if args.iters is not None:
        w["iters"] = args.iters
        w["desc"] += f" [profiling run: {args.iters} iterations]"
    if args.only:
        run_phase(args, w)
    elif args.impl == "reference":
        run_reference(args, w, rank, world)
    else:
        run_ours(args, w, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
