#!/usr/bin/env python3
"""Benchmark: MarchingCubesSearch of the 48-minus-16 CSG tree (delta 0.004,
iters 8) on one GB300 — corners/s of the FP32-filtered kernel, next to the
plain FP64 kernel (bit-identical meshes) and the CPU restatement of the
reference path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one MarchingCubesSearch of the solid resident on the device
(corner classification, cube classification + prefix sums, emission, edge
bisection).  L2 is flushed (a 256 MiB write) before every timed step; step
time is the library's CUDA-event time on its own stream.  Under torchrun
every rank meshes the headline solid (weak scaling: one solid a rank) and
``value`` sums all ranks' corners over the slowest rank's time; the batched
configurations (512 CSG solids, 64 colliders) are split across the ranks by
solid, largest first (model3d_gb300/shard.py), with no collective on the
data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "corners/sec & meshes/sec: FP32-filtered vs FP64 GPU, bit-identical mesh"
WORKLOAD = "csg_tree(seed=1, 48 joined primitives minus 16), delta=0.004, iters=8"
SEED, N_POS, N_NEG, DELTA, ITERS = 1, 48, 16, 0.004, 8
L2_NOTE = "inputs resident in HBM; the GPU arm flushes L2 (256 MiB write) before every timed step"


def workload_config(grid):
    """The `config` of both arms (identical, so the two lines describe the same
    workload): the solid, the spacer grid and its corner count."""
    nx, ny, nz = (int(v) for v in grid)
    return {"workload": WORKLOAD, "grid": [nx, ny, nz], "corners": nx * ny * nz, "l2": L2_NOTE}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_sample(nodes, sets, threads):
    """The oracle over the whole grid of the workload: the C++ restatement of
    the reference path (slab scan, cube pass, bisection search), on `threads`
    host threads."""
    from oracle import oracle as O
    t = time.perf_counter()
    m = O.mc_search(nodes, sets, DELTA, ITERS, threads=threads)
    dt = time.perf_counter() - t
    corners = m["nx"] * m["ny"] * m["nz"]
    return corners / dt, dict(grid=(m["nx"], m["ny"], m["nz"]), corners=corners, seconds=dt,
                              triangles=len(m["tris"]), leaf_evals=m["leaf_evals"])


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from model3d_gb300 import serialize
    from model3d_gb300.workloads import csg_tree
    solid = csg_tree(SEED, N_POS, N_NEG)
    nodes, sets = serialize(solid)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(nodes, sets, threads)
    secs, info = [], None
    for _ in range(args.steps):
        _, info = cpu_sample(nodes, sets, threads)
        secs.append(info["seconds"])
    ms_step = 1000 * float(np.mean(secs))
    value = info["corners"] / (ms_step / 1000.0)
    sample = (f"oracle port (C++ restatement of model3d MarchingCubesSearch; no Go toolchain), "
              f"{threads} threads, the whole {info['grid'][0]} x {info['grid'][1]} x {info['grid'][2]} grid "
              f"per step (slab scan, cube pass and bisection search)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "corners/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded splitmix64)",
        "config": workload_config(info["grid"]),
        "precision": "fp64 (CPU)",
        "meshes_per_s": 1000.0 / ms_step,
        "cpu_baseline": {"value": value, "unit": "corners/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "corners/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from model3d_gb300 import (Context, DeviceSolid, MarchingCubesSearch, serialize)
    from model3d_gb300 import _native as N
    from model3d_gb300.workloads import csg_tree
    import ctypes

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    ctx = Context(local)
    solid = csg_tree(SEED, N_POS, N_NEG)
    ds = DeviceSolid(solid, ctx)
    L = N.lib()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def step(prec):
        o = N.MCOpts()
        o.precision = prec
        o.cull = 1
        V, T = ctypes.c_int64(), ctypes.c_int64()
        st = N.MCStats()
        s = L.mc_search_device(ctx.ptr, ds.ptr, DELTA, ITERS, ctypes.byref(o), ctypes.byref(V),
                               ctypes.byref(T), ctypes.byref(st))
        if s != 0:
            raise RuntimeError(L.mc_last_error(ctx.ptr).decode())
        return st.as_dict()

    def timed(prec, K):
        sts = []
        for _ in range(K):
            flush.zero_()
            torch.cuda.synchronize()
            sts.append(step(prec))
        return sts

    # Tile shape chosen by the library's autotuner (outside the timed region).
    from model3d_gb300 import autotune, measure_peaks
    tuned = autotune(ds, DELTA, ITERS, ctx=ctx)
    for _ in range(args.warmup):
        step(N.MC_PREC_FP32_FILTERED)
        step(N.MC_PREC_FP64)

    # Bit-identity of the two precisions on this workload (same vertex and
    # triangle layout by construction, so array equality is mesh equality).
    def fetch():
        V, T = ctypes.c_int64(), ctypes.c_int64()
        st = step_stats[-1]
        v = np.zeros((st["vertices"], 3))
        t = np.zeros((st["triangles"], 3), dtype=np.int32)
        L.mc_result_copy(ctx.ptr, v.ctypes.data, t.ctypes.data)
        return v, t

    step_stats = [step(N.MC_PREC_FP32_FILTERED)]
    v32, t32 = fetch()
    step_stats.append(step(N.MC_PREC_FP64))
    v64, t64 = fetch()
    identical = bool(np.array_equal(v32.view(np.uint64), v64.view(np.uint64)) and
                     np.array_equal(t32, t64))

    barrier()
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        sts = timed(N.MC_PREC_FP32_FILTERED, args.steps)
    barrier()
    wall = time.perf_counter() - t0
    sts64 = timed(N.MC_PREC_FP64, args.steps)

    ms = [s["ms_total"] for s in sts]
    corners = sts[0]["corners"]
    ms_step, value = replica_rate(float(np.mean(ms)), corners, ws, "cuda")
    ms64 = float(np.mean([s["ms_total"] for s in sts64]))
    value64 = ws * corners / (ms64 / 1000.0)

    # End to end through the public call: serialise, lower + upload the solid,
    # search, copy the indexed mesh to host arrays.
    e2e_t, h2d, d2h = [], 0, 0
    for i in range(max(args.steps, 1)):
        torch.cuda.synchronize()
        t = time.perf_counter()
        m = MarchingCubesSearch(solid, DELTA, ITERS, ctx=ctx)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t)
        h2d = m.stats["h2d_bytes"] + int(ds.nodes.nbytes)
        d2h = m.stats["d2h_bytes"]
    e2e_s = float(np.median(e2e_t))

    # Roofline of the dominant kernel.
    pk = measure_peaks(ctx)
    phases = {k: float(np.mean([s[k] for s in sts]))
              for k in ("ms_classify", "ms_count", "ms_emit", "ms_search")}
    dom = max(phases, key=phases.get)
    peaks, kind = measured_peaks()
    roof = roofline(dom, phases[dom], sts[0], peaks, kind, pk[0])

    others = {} if args.no_extra else other_configs(ctx, torch, flush, value, args.collider_batch)

    if rank == 0:
        cpu = None
        if ws == 1 and not args.no_cpu:
            threads = os.cpu_count() or 1
            nodes, sets = serialize(solid)
            cv, info = cpu_sample(nodes, sets, threads)
            cpu = {"value": cv, "unit": "corners/s", "cores": threads, "kind": "port",
                   "sample": (f"oracle port, {threads} threads, one run over the whole grid "
                              f"({info['corners']} corners, {info['seconds']:.1f} s)")}
        s0 = sts[0]
        alu = alu_roofline(s0, phases["ms_classify"] + phases["ms_search"], pk[0], info if cpu else None)
        out = {
            "metric": METRIC, "value": value, "unit": "corners/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-filtered/f64", "data": "synthetic (seeded splitmix64)",
            "config": workload_config((s0["nx"], s0["ny"], s0["nz"])),
            "precision": "fp32-filtered, fp64 escalation",
            "parallelism": "replicas" if ws > 1 else "1 GPU",
            "meshes_per_s": ws / (ms_step / 1000.0),
            "triangles_per_s": ws * s0["triangles"] / (ms_step / 1000.0),
            "fp64": {"value": value64, "unit": "corners/s", "ms_per_step": ms64},
            "fp32_over_fp64": value / value64,
            "bit_identical_fp32_fp64": identical,
            "escalation_rate": s0["escalations"] / max(1, s0["leaf_evals"]),
            "mesh": {"vertices": s0["vertices"], "triangles": s0["triangles"]},
            "phases_ms": phases,
            "gpu_launches": 6 * args.steps,
            "roofline": roof,
            "tiles": {"tile_y": tuned[0], "tile_z": tuned[1], "chosen_by": "mc_autotune"},
            "measured_peaks_this_gpu": {"fp32_tflops": pk[0], "fp64_tflops": pk[1], "l2_read_gbs": pk[2]},
            "alu_roofline": alu,
            "other_configs": others,
            "clocks": clk.summary(),
            "wall_s_timed_region": wall,
            "e2e": {"value": corners / e2e_s, "unit": "corners/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": 1000 * e2e_s},
            "cpu_baseline": cpu,
        }
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def replica_rate(ms_step, corners, ws, device):
    """Whole-job rate of ws independent replicas: every rank processed
    `corners` per step; the step time is the slowest rank's (all_reduce MAX
    over the process group, any backend).  Returns (ms_step, corners/s)."""
    if ws > 1:
        import torch
        t = torch.tensor([ms_step], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_step = float(t.item())
    return ms_step, ws * corners / (ms_step / 1000.0)


def _device_rate(L, N, ctx, ds, delta, iters, prec, flush, torch, reps=3):
    import ctypes
    o = N.MCOpts()
    o.precision = prec
    o.cull = 1
    V, T = ctypes.c_int64(), ctypes.c_int64()
    best = None
    for _ in range(reps + 1):
        flush.zero_()
        torch.cuda.synchronize()
        st = N.MCStats()
        if L.mc_search_device(ctx.ptr, ds.ptr, delta, iters, ctypes.byref(o), ctypes.byref(V),
                              ctypes.byref(T), ctypes.byref(st)) != 0:
            raise RuntimeError(L.mc_last_error(ctx.ptr).decode())
        d = st.as_dict()
        if best is None or d["ms_total"] < best["ms_total"]:
            best = d
    return best


def other_configs(ctx, torch, flush, single_rate, count=16):
    """The other benchmark configurations, device time (CUDA events, best of 3
    after a warm-up): unit sphere (delta 0.01), the 1,048,820-triangle
    displaced icosphere collider on a ~256^3 grid, 512 CSG solids in one
    batched launch (graph replay) next to the same solids one call at a
    time, a 64-ball metaball, batched colliders, and SaveGroupedSTL of the
    headline mesh (wall time, host bytes out).  A configuration that
    fails is reported under its name with the error, without losing the
    others or the headline line."""
    out = {}
    lines = [("sphere_r1_delta0.01", lambda: sphere_line(ctx, torch, flush)),
             ("collider_icosphere_1048820_tris_256cubed", lambda: collider_line(ctx, torch, flush)),
             ("batch_512_csg", lambda: batch_line(ctx, torch, flush, single_rate)),
             ("metaball_blob64_quartic_delta0.005", lambda: metaball_line(ctx, torch, flush)),
             ("batch_colliders", lambda: collider_batch_line(ctx, count, torch)),
             ("save_grouped_stl_headline", lambda: grouped_stl_line(ctx, torch))]
    for name, f in lines:
        try:
            out.update(f())
        except Exception as e:  # noqa: BLE001 - reported in the JSON line
            out[name] = {"error": f"{type(e).__name__}: {e}"[:300]}
    return out


def grouped_stl_line(ctx, torch):
    """SaveGroupedSTL of the headline mesh (4.17M triangles): GroupTriangles
    and the STL encoding on the device over the search result, bytes copied
    to the host (wall time, best of 3 after a warm-up), next to the plain
    EncodeSTL of the same result; end to end from the resident solid
    (search + group + encode + copy into a reused buffer); and the Python
    call MarchingCubesSearchGroupedSTL, whose fresh 208 MB buffer is
    page-faulted on every call."""
    import ctypes
    import time
    import numpy as np
    from model3d_gb300 import DeviceSolid, MarchingCubesSearchGroupedSTL
    from model3d_gb300 import _native as N
    from model3d_gb300.workloads import csg_tree
    L = N.lib()
    ds = DeviceSolid(csg_tree(SEED, N_POS, N_NEG), ctx)
    o = N.MCOpts()
    o.precision = N.MC_PREC_FP32_FILTERED
    o.cull = 1
    V, T = ctypes.c_int64(), ctypes.c_int64()
    st = N.MCStats()
    if L.mc_search_device(ctx.ptr, ds.ptr, DELTA, ITERS, ctypes.byref(o), ctypes.byref(V), ctypes.byref(T),
                          ctypes.byref(st)) != 0:
        raise RuntimeError(L.mc_last_error(ctx.ptr).decode())
    n = ctypes.c_size_t()
    L.mc_result_stl(ctx.ptr, None, 0, ctypes.byref(n))
    buf = np.empty(n.value, dtype=np.uint8)

    def wall(f, reps=3):
        best = None
        for _ in range(reps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            f()
            dt = (time.perf_counter() - t0) * 1e3
            best = dt if best is None else min(best, dt)
        return best

    def call(fn):
        if fn(ctx.ptr, buf.ctypes.data, n.value, ctypes.byref(n)) != 0:
            raise RuntimeError(L.mc_last_error(ctx.ptr).decode())

    def search_group():
        s2 = N.MCStats()
        if L.mc_search_device(ctx.ptr, ds.ptr, DELTA, ITERS, ctypes.byref(o), ctypes.byref(V), ctypes.byref(T),
                              ctypes.byref(s2)) != 0:
            raise RuntimeError(L.mc_last_error(ctx.ptr).decode())
        call(L.mc_result_stl_grouped)

    ms_grouped = wall(lambda: call(L.mc_result_stl_grouped))
    ms_plain = wall(lambda: call(L.mc_result_stl))
    ms_e2e = wall(search_group)
    ms_py = wall(lambda: MarchingCubesSearchGroupedSTL(ds, DELTA, ITERS, ctx=ctx), reps=1)
    return {"save_grouped_stl_headline": {
        "triangles": T.value, "stl_bytes": n.value,
        "ms_group_encode_copy": ms_grouped, "ms_plain_encode_copy": ms_plain,
        "ms_search_group_encode_copy": ms_e2e,
        "ms_python_call_fresh_buffer": ms_py,
        "triangles_per_s_grouped": T.value / (ms_grouped / 1e3)}}


def sphere_line(ctx, torch, flush):
    from model3d_gb300 import DeviceSolid, Sphere, XYZ
    from model3d_gb300 import _native as N
    L = N.lib()
    sph = DeviceSolid(Sphere(XYZ(0, 0, 0), 1.0), ctx)
    a = _device_rate(L, N, ctx, sph, 0.01, 8, N.MC_PREC_FP32_FILTERED, flush, torch)
    b = _device_rate(L, N, ctx, sph, 0.01, 8, N.MC_PREC_FP64, flush, torch)
    return {"sphere_r1_delta0.01": {"corners": a["corners"], "triangles": a["triangles"],
                                    "fp32_corners_per_s": a["corners"] / (a["ms_total"] / 1e3),
                                    "fp64_corners_per_s": b["corners"] / (b["ms_total"] / 1e3),
                                    "ms_fp32": a["ms_total"], "ms_fp64": b["ms_total"]}}


def collider_line(ctx, torch, flush):
    from model3d_gb300 import DeviceSolid, MeshToCollider, NewColliderSolid
    from model3d_gb300 import _native as N
    from model3d_gb300.workloads import displaced_icosphere
    L = N.lib()
    tris = displaced_icosphere(229)
    col = NewColliderSolid(MeshToCollider(tris))
    mn, mx = col.Min(), col.Max()
    d = max(mx.X - mn.X, mx.Y - mn.Y, mx.Z - mn.Z) / 255
    t0 = time.perf_counter()
    cds = DeviceSolid(col, ctx)
    lower_s = time.perf_counter() - t0
    a = _device_rate(L, N, ctx, cds, d, 8, N.MC_PREC_FP32_FILTERED, flush, torch, reps=2)
    b = _device_rate(L, N, ctx, cds, d, 8, N.MC_PREC_FP64, flush, torch, reps=1)
    tests = a["bvh_nodes"] + a["bvh_tris"]
    # End to end through MarchingCubesSearch with host arrays: from the host
    # triangles (MeshToCollider's lowering: grouping, tree, ray grid; upload;
    # search; mesh copied back), and with the lowered solid resident.
    from model3d_gb300 import MarchingCubesSearch
    full, resident, m = [], [], None
    for _ in range(3):
        torch.cuda.synchronize()
        t = time.perf_counter()
        m = MarchingCubesSearch(col, d, 8, ctx=ctx)
        torch.cuda.synchronize()
        full.append(time.perf_counter() - t)
        t = time.perf_counter()
        m = MarchingCubesSearch(cds, d, 8, ctx=ctx)
        torch.cuda.synchronize()
        resident.append(time.perf_counter() - t)
    e2e = {"from_host_triangles_ms": 1e3 * float(np.median(full)),
           "solid_resident_ms": 1e3 * float(np.median(resident)),
           "corners_per_s_from_host_triangles": a["corners"] / float(np.median(full)),
           "corners_per_s_solid_resident": a["corners"] / float(np.median(resident)),
           "h2d_bytes_solid": int(sum(t.nbytes for t in [tris]) + cds.nodes.nbytes),
           "d2h_bytes": int(m.stats["d2h_bytes"])}
    return {"collider_icosphere_1048820_tris_256cubed": {
        "grid": [a["nx"], a["ny"], a["nz"]], "triangles_in": len(tris), "triangles_out": a["triangles"],
        "fp32_corners_per_s": a["corners"] / (a["ms_total"] / 1e3),
        "fp64_corners_per_s": b["corners"] / (b["ms_total"] / 1e3),
        "ms_fp32": a["ms_total"], "ms_fp64": b["ms_total"],
        "escalation_rate": a["escalations"] / max(1, tests), "bvh_box_tests": a["bvh_nodes"],
        "triangle_tests": a["bvh_tris"], "host_lowering_s": lower_s, "e2e": e2e}}


def rank_share(jobs, torch):
    """Under torchrun: this rank's jobs of a largest-first partition by
    corner count (model3d_gb300/shard.py), and a function that turns this
    rank's (ms, corners) into the whole job's (slowest rank's ms, all
    corners).  One process: all jobs, identity."""
    ws, rank, _ = dist_env()
    if ws == 1:
        return jobs, (lambda ms, corners: (ms, corners)), "1 GPU"
    from model3d_gb300.shard import job_costs, partition_jobs
    mine = partition_jobs(job_costs(jobs), ws)[rank]

    def combine(ms, corners):
        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        c = torch.tensor([float(corners)], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(c, op=torch.distributed.ReduceOp.SUM)
        return float(t.item()), int(c.item())

    return [jobs[i] for i in mine], combine, f"{ws} GPUs, jobs split largest-first by corners"


def batch_line(ctx, torch, flush, single_rate):
    from model3d_gb300 import DeviceSolid, MarchingCubesSearchBatch
    from model3d_gb300 import _native as N
    from model3d_gb300.workloads import csg_batch
    L = N.lib()
    items = csg_batch(2024, count=512)
    jobs, combine, par = rank_share([(DeviceSolid(s, ctx), dd, 8) for s, dd in items], torch)
    res = {}
    for prec in ("fp32", "fp64"):
        ms = []
        for _ in range(4):
            m = MarchingCubesSearchBatch(jobs, precision=prec, ctx=ctx)
            ms.append(m[0].stats["ms_total"])
        res[prec] = (min(ms[1:]), sum(x.stats["corners"] for x in m), sum(x.NumTriangles() for x in m))
    seq, big = 0.0, None
    for ds_, dd, it in jobs:
        r = _device_rate(L, N, ctx, ds_, dd, it, N.MC_PREC_FP32_FILTERED, flush, torch, reps=0)
        seq += r["ms_total"]
        if big is None or r["corners"] > big[1]["corners"]:
            big = ((ds_, dd, it), r)
    (bds, bd, bit), _ = big
    br = _device_rate(L, N, ctx, bds, bd, bit, N.MC_PREC_FP32_FILTERED, flush, torch, reps=3)
    big_rate = br["corners"] / (br["ms_total"] / 1e3)
    ms32, corners = combine(res["fp32"][0], res["fp32"][1])
    ms64, _ = combine(res["fp64"][0], res["fp64"][1])
    res["fp32"] = (ms32, corners, res["fp32"][2])
    res["fp64"] = (ms64, corners, res["fp64"][2])
    return {"batch_512_csg": {
        "jobs": len(items), "parallelism": par, "corners": corners, "triangles": res["fp32"][2],
        "fp32_corners_per_s": corners / (res["fp32"][0] / 1e3),
        "fp32_meshes_per_s": len(items) / (res["fp32"][0] / 1e3),
        "fp64_corners_per_s": corners / (res["fp64"][0] / 1e3),
        "ms_fp32_graph_replay": res["fp32"][0], "ms_fp64_graph_replay": res["fp64"][0],
        "sequential_single_calls_ms": seq,
        "batched_over_sequential": seq / res["fp32"][0],
        "fraction_of_single_large_solid_rate": (corners / (res["fp32"][0] / 1e3)) / single_rate,
        "largest_job_alone": {"corners": br["corners"], "triangles": br["triangles"],
                              "fp32_corners_per_s": big_rate},
        "fraction_of_largest_job_alone_rate": (corners / (res["fp32"][0] / 1e3)) / big_rate}}


def metaball_line(ctx, torch, flush):
    """A 64-ball quartic MetaballSolid (metaball_blob(3, 64), 3/4 spheres and
    1/4 capsules) at delta 0.005, FP32-filtered against FP64, with the two
    precisions' meshes compared bit for bit."""
    from model3d_gb300 import DeviceSolid, MarchingCubesSearch, canonical
    from model3d_gb300 import _native as N
    from model3d_gb300.workloads import metaball_blob
    L = N.lib()
    ds = DeviceSolid(metaball_blob(3, 64), ctx)
    a = _device_rate(L, N, ctx, ds, 0.005, 8, N.MC_PREC_FP32_FILTERED, flush, torch, reps=2)
    b = _device_rate(L, N, ctx, ds, 0.005, 8, N.MC_PREC_FP64, flush, torch, reps=1)
    m32 = MarchingCubesSearch(ds, 0.005, 8, precision="fp32", ctx=ctx)
    m64 = MarchingCubesSearch(ds, 0.005, 8, precision="fp64", ctx=ctx)
    same = bool(np.array_equal(canonical(m32.TriangleSoup()), canonical(m64.TriangleSoup())))
    return {"metaball_blob64_quartic_delta0.005": {
        "grid": [a["nx"], a["ny"], a["nz"]], "balls": 64, "triangles": a["triangles"],
        "fp32_corners_per_s": a["corners"] / (a["ms_total"] / 1e3),
        "fp64_corners_per_s": b["corners"] / (b["ms_total"] / 1e3),
        "ms_fp32": a["ms_total"], "ms_fp64": b["ms_total"],
        "phases_ms_fp32": {k: a[k] for k in ("ms_classify", "ms_count", "ms_emit", "ms_search")},
        "escalation_rate": a["escalations"] / max(1, a["leaf_evals"]),
        "bit_identical_fp32_fp64": same}}


def collider_batch_line(ctx, count, torch):
    """Displaced-icosphere colliders (triangles log-uniform in [20k, 2M], grid
    sides log-uniform in [128, 512]) meshed in one batched launch, FP32-filtered
    (graph replay) and FP64, with the two precisions' meshes compared."""
    from model3d_gb300 import (DeviceSolid, MarchingCubesSearchBatch, MeshToCollider,
                               NewColliderSolid)
    from model3d_gb300.workloads import collider_batch
    if count <= 0:
        return {}
    t0 = time.perf_counter()
    meshes = collider_batch(77, count=count)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    jobs = []
    for tris, _, side in meshes:
        s = NewColliderSolid(MeshToCollider(tris))
        mn, mx = s.Min(), s.Max()
        ext = max(mx.X - mn.X, mx.Y - mn.Y, mx.Z - mn.Z)
        jobs.append((DeviceSolid(s, ctx), ext / (side - 3), 8))
    lower_s = time.perf_counter() - t0
    jobs, combine, par = rank_share(jobs, torch)
    ms = {}
    outs = {}
    for prec, reps in (("fp32", 3), ("fp64", 1)):
        times = []
        for _ in range(reps):
            m = MarchingCubesSearchBatch(jobs, precision=prec, ctx=ctx)
            bad = [x for x in m if not hasattr(x, "stats")]
            if bad:
                raise RuntimeError(f"collider batch job failed: {bad[0]}")
            times.append(m[0].stats["ms_total"])
        ms[prec] = min(times[1:]) if len(times) > 1 else times[0]
        outs[prec] = m
    same = all(np.array_equal(a.vertices.view(np.uint64), b.vertices.view(np.uint64)) and
               np.array_equal(a.triangles, b.triangles) for a, b in zip(outs["fp32"], outs["fp64"]))
    corners = sum(x.stats["corners"] for x in outs["fp32"])
    ms["fp32"], all_corners = combine(ms["fp32"], corners)
    ms["fp64"], _ = combine(ms["fp64"], corners)
    corners = all_corners
    st0 = outs["fp32"][0].stats  # counters of a batched launch are batch totals
    tests = st0["bvh_tris"] + st0["bvh_nodes"]
    esc = st0["escalations"]
    name = f"batch_{count}_colliders" + ("" if count == 64 else "_of_the_64_mesh_configuration")
    return {name: {
        "jobs": count, "parallelism": par, "triangles_in": int(sum(len(t) for t, _, _ in meshes)),
        "corners": corners, "triangles_out": sum(x.NumTriangles() for x in outs["fp32"]),
        "fp32_corners_per_s": corners / (ms["fp32"] / 1e3),
        "fp64_corners_per_s": corners / (ms["fp64"] / 1e3),
        "ms_fp32_graph_replay": ms["fp32"], "ms_fp64": ms["fp64"],
        "bit_identical_fp32_fp64": bool(same),
        "escalation_rate": esc / max(1, tests),
        "host_generate_s": gen_s, "host_lower_s": lower_s}}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# each kernel on this workload, from the ncu capture of the full-size grid
# summarised in profiles/launches_csg48_delta0.004.md (same kernels as this
# source).  Below the algorithmic bytes where a kernel reads what the previous
# one left in the 129 MB L2 (keys, corner bits) or its writes stay in L2.
NCU_TRAFFIC = {"k_count": 29754624, "k_emit": 50758656, "k_search": 45146880}


def algorithmic_bytes(kernel, st):
    """Bytes a kernel must move per launch: corner bits, chunk counts and
    offsets, keys, vertices and triangles."""
    nx, ny, nz = st["nx"], st["ny"], st["nz"]
    W = (nx + 31) // 32 + 1
    bits = nz * ny * W * 4
    chunks = ((nx - 1 + 31) // 32) * (ny - 1) * (nz - 1)
    V, T = st["vertices"], st["triangles"]
    if kernel == "k_classify":
        return bits                                  # one bit per corner written
    if kernel == "k_count":
        return bits + chunks * 4 * 3                 # bits read; counts + 2 prefixes written
    if kernel == "k_emit":
        return bits + chunks * 12 + V * 8 + T * 12   # bits + offsets read; keys, triangles written
    return V * 8 + V * 24                            # keys read, vertices written


def roofline(kernel, ms, st, peaks, kind, fp32_tflops):
    """The dominant kernel against the bound that limits it.  Classification
    and search evaluate leaf predicates: their bound is the FP32 ALU, and
    `achieved` is the float operations of the reference formulas of the
    leaves they evaluated (their own device counter, weighted by kind) over
    the kernel's event time, against the FP32 peak measured on this GPU.  The
    HBM figures of the same launch ride along under `hbm`.  Count, scan and
    emission are bound by HBM / L2 and report against the measured copy
    bandwidth."""
    name = kernel.replace("ms_", "k_")
    alg = algorithmic_bytes(name, st)
    gbs = alg / (ms / 1000.0) / 1e9
    peak_hbm = float(peaks.get("hbm_gbs", 6800.0))
    hbm = {"achieved": gbs, "peak": peak_hbm, "unit": "GB/s", "frac": gbs / peak_hbm,
           "algorithmic_bytes": int(alg), "traffic": NCU_TRAFFIC.get(name), "peak_kind": kind}
    if name in ("k_classify", "k_search"):
        flops = st["flops_search" if name == "k_search" else "flops_classify"]
        tf = flops / (ms / 1000.0) / 1e12
        return {"kernel": name, "bound": "alu_fp32", "achieved": tf, "peak": fp32_tflops, "unit": "TFLOP/s",
                "frac": tf / fp32_tflops, "traffic": NCU_TRAFFIC.get(name), "flops": int(flops), "ms": ms,
                "peak_kind": "measured on this GPU (mc_measure_peaks: dense FP32 FMA loop)", "hbm": hbm}
    return {"kernel": name, "bound": "hbm", "achieved": gbs, "peak": peak_hbm, "unit": "GB/s",
            "frac": gbs / peak_hbm, "traffic": NCU_TRAFFIC.get(name), "algorithmic_bytes": int(alg), "ms": ms,
            "peak_kind": kind}


def alu_roofline(st, ms, fp32_tflops, ref=None):
    """Float operations of the reference formulas of the leaves that the
    classification and search kernels evaluated (their device counters,
    weighted by kind: Sphere 10, Rect 6, Cylinder and Capsule 23, Torus 36)
    over those kernels' event time, against the measured FP32 peak.  With
    ref (the oracle's leaf evaluations per corner over the same grid) it adds
    the operations of the reference's short-circuit evaluation of the whole
    grid, over the same time: tile culling skips most of them."""
    flops = st["flops_classify"] + st["flops_search"]
    achieved = flops / (ms / 1000.0) / 1e12
    per_leaf = flops / max(1, st["leaf_evals"])
    out = {"bound": "fp32_alu", "kernels": ["k_classify", "k_search"], "achieved": achieved,
           "peak": fp32_tflops, "unit": "TFLOP/s", "frac": achieved / fp32_tflops,
           "leaf_evals": int(st["leaf_evals"]), "flops": int(flops), "flops_per_leaf_eval": per_leaf, "ms": ms,
           "peak_kind": "measured on this GPU (mc_measure_peaks)"}
    if ref:
        ref_flops = ref["leaf_evals"] / ref["corners"] * st["corners"] * per_leaf
        out["reference_work"] = {"leaf_evals_per_corner": ref["leaf_evals"] / ref["corners"],
                                 "flops": ref_flops, "tflops_equivalent": ref_flops / (ms / 1000.0) / 1e12}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extra", action="store_true", help="skip the other configurations")
    ap.add_argument("--collider-batch", type=int, default=64,
                    help="meshes in the batched-collider line (64 = the full configuration)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
