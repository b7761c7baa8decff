"""Benchmark: uniform-grid isosurface extraction on one GB300 (replicas on N GPUs).

Workload (default): the 512^3 dense-ambiguity field -- a 33^3 grid of U[-1,1] values (seeded)
trilinearly upsampled to 512^3 plus 0.02*N(0,1) per voxel, isovalue 0 -- extracted each step
with TMC (shared-vertex triangles) and with DMC (halfedges, triangles, P3X3Y colour + isolated +
P3333 simplification).  Synthetic data (no datasets exist for this path).  The field (512 MiB) is
larger than L2, so no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
    python bench.py --grid 320 --steps 1 --warmup 1 --no-cpu-baseline   # small case for profiling
    python bench.py --workload batch          # 256 uneven volumes: one batched call vs 256 plain calls
    python bench.py --workload precision      # 1024^3 seeded saddles: topology vs the oracle, position error
    python bench.py --workload serve          # Poisson request stream: server vs one call per request
    python bench.py --workload plain64        # the 64^3 Gaussian-blob plain DMC call (latency-bound)
    python bench.py --workload fused          # generated 512^3 fields: stored vs fused generation

Prints one JSON line.  `value` is device-resident throughput (field already in HBM); `e2e` is the
same metric through the C ABI with host buffers (field copied in, mesh copied out every step).
The default line also carries `batch` (the 256-volume batched workload: one batched call against
256 plain calls) and `serve` (Poisson arrivals at 0.5x and 1.5x the plain loop's capacity: the
server's p50/p99 latency and Gcells/s against one call per request); --no-extras leaves them out.
Cells per step = 511^3: each step extracts the one volume with both algorithms, and its cells are
counted once (the CPU baseline and the reference arm count the same way).
"""
from __future__ import annotations

import argparse
import concurrent.futures
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gcells/s"
N = 512
SEED = 1


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--grid", type=int, default=N, help="points per axis of the noise field (profiling cases)")
    p.add_argument("--workload", default="single", choices=["single", "batch", "precision", "serve", "plain64", "fused"],
                   help="single: the 512^3 volume (TMC + DMC); batch: 256 uneven volumes, DMC; "
                        "precision: 1024^3 periodic field with seeded near-singular saddles")
    p.add_argument("--volumes", type=int, default=256, help="volumes of the batch workload")
    p.add_argument("--requests", type=int, default=256, help="requests per arrival rate of the serve workload")
    p.add_argument("--rates", default="0.5,0.8,1.0,1.5",
                   help="arrival rates of the serve workload, as multiples of the plain loop's capacity")
    p.add_argument("--in-flight", type=int, default=3,
                   help="end-to-end steps in flight at once (each on its own pair of contexts)")
    p.add_argument("--no-extras", action="store_true",
                   help="default workload only, without the batch and serve keys")
    return p.parse_args()


def dist_env():
    from tmc_gb300.replicas import dist_env as env
    return env()


# ------------------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) > 8:
                for i, nm in enumerate(names):
                    if r[5 + i].lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# ------------------------------------------------------------------------------------------------
# our arm
# ------------------------------------------------------------------------------------------------
# Kernel groups of the roofline: the profiler stages of one piece of work, and the DRAM traffic per
# algorithmic byte that ncu measured for them on the 320^3 case of this workload (profiles/
# dmc_vertex_noise320.md: 2,772 MB for 5.49 M vertices; tmc_emit_noise320.md: 1,189 MB for 267.7 MB of
# mesh; classify_noise320.md: 218.2 MB for a 131.1 MB field), scaled to the full launch by the units
# it processes (traffic grows with the vertex / cell count).
ROOFLINE_GROUPS = {
    "dmc_vertex": (("dmc_vertex_setup", "dmc_project", "dmc_vertex_finish", "dmc_vertex"), 2771.6 / 131.6),
    "dmc_halfedges": (("dmc_halfedges",), None),
    "tmc_emit": (("tmc_emit",), 1188.9 / 267.7),
    "dmc_classify": (("dmc_classify",), 218.2 / 131.1),
    "tmc_classify": (("tmc_classify",), None),
    "dmc_quad": (("dmc_quad",), None),
    "dmc_triangles": (("dmc_triangles",), None),
}


def link_bandwidth(torch) -> dict:
    """Host link bandwidth right now: a pinned 256 MiB buffer copied in and out (best of three each,
    CUDA events), in GB/s.  The link is shared with the other GPUs of the machine, so the end-to-end
    figure is read against it."""
    n = 64 << 20
    h = torch.empty(n, dtype=torch.float32).pin_memory()
    d = torch.empty(n, dtype=torch.float32, device="cuda")
    out = {}
    for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
        best = 0.0
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            best = max(best, 4 * n / (e0.elapsed_time(e1) * 1e-3) / 1e9)
        out[name] = round(best, 1)
    del h, d
    return out


def algorithmic_bytes(group: str, sizes: dict, cells: int, voxels: int) -> float:
    """Algorithmic bytes of one launch of a kernel group: the field read once (4 B/voxel) for the
    classifying kernels, the mesh bytes a group emits for the others (24 B/vertex, 16 B/quad,
    12 B/triangle, 16 B/halfedge + 4 B/vertex + 4 B/face); scratch and re-reads excluded."""
    if group in ("tmc_classify", "dmc_classify"):
        return 4.0 * voxels
    if group == "tmc_emit":
        return 24.0 * sizes["tmc_v"] + 12.0 * sizes["tmc_t"]
    if group == "dmc_vertex":
        return 24.0 * sizes["dmc_front_v"]
    if group == "dmc_quad":
        return 16.0 * sizes["dmc_front_q"]
    if group == "dmc_halfedges":
        return 16.0 * sizes["dmc_he"] + 4.0 * sizes["dmc_v"] + 4.0 * sizes["dmc_q"]
    if group == "dmc_triangles":
        return 12.0 * sizes["dmc_t"]
    return 0.0


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    from tmc_gb300 import native, volumes
    try:
        native.load()
    except RuntimeError:
        from tmc_gb300 import build
        build.build()
    from tmc_gb300.replicas import Replicas, replica_seed, reports, throughput
    torch.cuda.set_device(local)
    rep = Replicas(world, "nccl", local)  # replicas: no collective on the data path
    n = args.grid
    vol = volumes.noise_volume(n, seed=replica_seed(SEED, rank))
    cells = vol.cells
    voxels = vol.data.size
    ctx = native.Context(local)
    dev = torch.from_numpy(vol.data).cuda()
    vdev = native.make_volume(vol, dev.data_ptr(), on_device=True)
    host = torch.from_numpy(vol.data).pin_memory()
    vhost = native.make_volume(vol, host.data_ptr(), on_device=False)
    stream = torch.cuda.ExternalStream(ctx.stream)
    dmc_flags = native.DMC_SIMPLIFY | native.OUT_HALFEDGES | native.OUT_TRIANGLES
    # The step's two extractions are independent: the TMC one runs on its own context (stream) from a
    # helper thread while this thread runs the DMC one, so their kernels share the GPU.
    ctx_t = native.Context(local)
    stream_t = torch.cuda.ExternalStream(ctx_t.stream)
    helper = concurrent.futures.ThreadPoolExecutor(1)

    def step(v, extra=0):
        ft = helper.submit(ctx_t.tmc_raw, v, vol.iso, extra)
        md = ctx.dmc_raw(v, vol.iso, dmc_flags | extra)
        return ft.result(), md

    def step_sequential(v, extra=0):  # both on one context, for the per-stage profile
        mt = ctx.tmc_raw(v, vol.iso, extra)
        md = ctx.dmc_raw(v, vol.iso, dmc_flags | extra)
        return mt, md

    def barrier():
        torch.cuda.synchronize()
        rep.barrier()

    max_over_ranks = rep.max_over_ranks

    sizes = {}
    for _ in range(args.warmup):
        mt, md = step(vdev)
        sizes = {"tmc_v": mt.nr_v, "tmc_t": mt.nr_t, "dmc_v": md.nr_v, "dmc_q": md.nr_q, "dmc_t": md.nr_t,
                 "dmc_he": md.nr_he}
        ctx_t.free(mt)
        ctx.free(md)
    # ---- device-resident timed region ----
    barrier()
    l0 = ctx.launches() + ctx_t.launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    et = torch.cuda.Event()
    with ClockSampler(local) as clk:
        e0.record(stream)
        stream_t.wait_event(e0)  # the TMC stream starts inside the timed region
        for _ in range(args.steps):
            mt, md = step(vdev)
            ctx_t.free(mt)
            ctx.free(md)
        et.record(stream_t)
        stream.wait_event(et)  # e1 follows the work of both streams
        e1.record(stream)
        barrier()
    launches = ctx.launches() + ctx_t.launches() - l0
    ms = max_over_ranks(e0.elapsed_time(e1))
    ms_step = ms / args.steps
    value = throughput(world, cells, args.steps, ms * 1e-3)
    # ---- end to end through the C ABI with host buffers (W untimed steps first) ----
    # With results going to host memory the link, not the GPU, sets the end of a step: the TMC
    # extraction runs on a context of higher stream priority (tmc_ctx_opts.priority), so that it
    # finishes early and its output crosses the link while DMC still computes.  A step's DMC meshes
    # exist only after its last pass, so their copy (about 10 ms of link time) is a tail that one
    # step cannot hide; with `--in-flight` steps in flight, each on its own pair of contexts driven
    # by its own thread (what a caller of the C ABI does from several threads), one step's meshes
    # cross the link while the next step computes.  Every step still copies its field in and its
    # meshes out inside the timed region.
    # The lanes run at different stream priorities: started together at one priority they would
    # compute at the same time and then copy out at the same time, leaving the link idle while they
    # compute and the GPU idle while they copy.  A higher lane finishes its compute first and copies
    # out while a lower one computes.  Measured at 512^3 (steps per second as Gcells/s): one lane
    # 3.87, two lanes at one priority 4.56, two at two priorities 4.43, three at one 4.65, three at
    # three 4.85, four at one 4.63.
    lanes = []
    nl = max(1, args.in_flight)
    for li in range(nl):
        pd = -2 * (nl - 1 - li)  # DMC context; the lane's TMC context one level above
        lanes.append({"dmc": native.Context(local, priority=pd), "tmc": native.Context(local, priority=pd - 1),
                      "helper": concurrent.futures.ThreadPoolExecutor(1),
                      "runner": concurrent.futures.ThreadPoolExecutor(1)})

    def step_lane(li):
        ln = lanes[li]
        ts = time.perf_counter()
        ft = ln["helper"].submit(ln["tmc"].tmc_raw, vhost, vol.iso, native.OUT_HOST)
        md = ln["dmc"].dmc_raw(vhost, vol.iso, dmc_flags | native.OUT_HOST)
        mt = ft.result()
        nbytes = (24 * mt.nr_v + 12 * mt.nr_t) + (24 * md.nr_v + 16 * md.nr_q + 12 * md.nr_t + 16 * md.nr_he +
                                                  4 * md.nr_v + 4 * md.nr_q)
        ln["tmc"].free(mt)
        ln["dmc"].free(md)
        return nbytes, round((time.perf_counter() - ts) * 1e3, 2)

    def run_steps(k, in_flight):
        futs = [lanes[q % in_flight]["runner"].submit(step_lane, q % in_flight) for q in range(k)]
        return [f.result() for f in futs]

    run_steps(max(1, args.warmup) * len(lanes), len(lanes))
    link_before = link_bandwidth(torch)
    # one step at a time: the line's e2e value (steady across runs)
    barrier()
    t0 = time.perf_counter()
    serial = run_steps(args.steps, 1)
    barrier()
    serial_s = max_over_ranks(time.perf_counter() - t0)
    # steps in flight (e2e.in_flight; host-load dependent): every lane runs the same number of steps, at least four, so
    # that the measurement covers the lanes' steady state rather than their start and a lone last step
    e2e_steps = len(lanes) * max(4, -(-args.steps // len(lanes)))
    barrier()
    t0 = time.perf_counter()
    res = run_steps(e2e_steps, len(lanes))
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    d2h = res[-1][0]
    step_ms = [r[1] for r in serial]
    e2e = throughput(world, cells, e2e_steps, e2e_s)
    e2e_serial = throughput(world, cells, args.steps, serial_s)
    for ln in lanes:
        ln["helper"].shutdown()
        ln["runner"].shutdown()
        ln["tmc"].close()
        ln["dmc"].close()
    link_after = link_bandwidth(torch)
    # ---- per-stage profile (separate pass, not timed above) ----
    ctx.set_profiling(True)
    m = ctx.dmc_raw(vdev, vol.iso, native.OUT_LOCAL)  # front end alone, for its mesh sizes
    sizes["dmc_front_v"], sizes["dmc_front_q"] = m.nr_v, m.nr_q
    ctx.free(m)
    ctx.set_profiling(True)
    for _ in range(2):
        mt, md = step_sequential(vdev)
        ctx.free(mt)
        ctx.free(md)
    prof = ctx.profile()
    ctx.set_profiling(False)
    total_ms = sum(v[0] for v in prof.values())
    # kernel groups (the vertex passes count as one), the dominant one by time
    groups = {}
    grouped = set()
    for gname, (members, _) in ROOFLINE_GROUPS.items():
        present = [m for m in members if m in prof]
        if present:
            groups[gname] = (sum(prof[m][0] for m in present), max(prof[m][1] for m in present))
            grouped.update(present)
    for k, v in prof.items():
        if k not in grouped:
            groups[k] = v
    dom_name, (dom_ms, dom_cnt) = max(groups.items(), key=lambda kv: kv[1][0])
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    avg_ms = dom_ms / max(dom_cnt, 1)
    algo = algorithmic_bytes(dom_name, sizes, cells, voxels)
    achieved = algo / (avg_ms * 1e-3) / 1e9 if algo else 0.0
    ratio = ROOFLINE_GROUPS.get(dom_name, ((), None))[1]
    traffic = round(ratio * algo) if (ratio and algo) else None
    stages = {k: {"ms_per_step": round(v[0] / 2, 4), "share": round(v[0] / total_ms, 4)} for k, v in prof.items()}
    # memory-bound classifier, reported beside the dominant kernel
    cls = {}
    for st in ("tmc_classify", "dmc_classify"):
        if st in prof:
            a = prof[st][0] / prof[st][1]
            cls[st] = {"ms": round(a, 4), "achieved_gbs": round(4.0 * voxels / (a * 1e-3) / 1e9, 1),
                       "frac": round(4.0 * voxels / (a * 1e-3) / 1e9 / peak, 4)}
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": "Gcells/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n}^3 noise field (33^3 U[-1,1] upsampled + 0.02 N(0,1)), isovalue 0: TMC shared-vertex"
                               " + DMC halfedge/triangles with P3X3Y+P3333 simplification per step",
                   "grid": [n, n, n], "cells_per_step": cells, "seed": SEED,
                   "l2": f"inputs larger than L2 ({4 * voxels / 2**20:.0f} MiB field)", "parallelism": f"replicas x{world}",
                   "streams": "the TMC and the DMC extraction of a step run concurrently, one context (stream) each; "
                              "in the end-to-end steps the TMC context has the higher stream priority (its output "
                              "then crosses the host link while DMC computes), and `in_flight` steps run at once, "
                              "each on its own pair of contexts and thread, so that one step's meshes cross the "
                              "link while the next computes; the stage profile and the roofline come from a "
                              "separate sequential pass"},
        "mesh": sizes,
        "e2e": {"value": round(e2e_serial, 4), "unit": "Gcells/s", "h2d_bytes_per_step": 2 * 4 * voxels,
                "d2h_bytes_per_step": int(d2h), "steps": args.steps,
                "ms_per_step": round(serial_s * 1e3 / args.steps, 3), "step_ms": step_ms,
                "in_flight": {"value": round(e2e, 4), "lanes": len(lanes), "steps": e2e_steps,
                              "ms_per_step": round(e2e_s * 1e3 / e2e_steps, 3),
                              "note": "the same steps with several in flight (lanes of contexts and threads at "
                                      "different stream priorities): one step's meshes cross the link while "
                                      "another computes; this throughput depends on the host's load (threads "
                                      "driving the lanes), so the line's value is the one-step-at-a-time one"},
                "host_link_gbs": {"before": link_before, "after": link_after,
                                  "note": "pinned 256 MiB copies each way, measured just before and after the "
                                          "end-to-end steps; the link is shared with the machine's other GPUs"}},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum on the 320^3 case, "
                                       "scaled by vertices" if traffic else None,
                     "algorithmic_bytes_per_launch": algo, "avg_launch_ms": round(avg_ms, 4),
                     "kernels": list(ROOFLINE_GROUPS.get(dom_name, ((dom_name,), None))[0]),
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6.8 TB/s"},
        "classify_roofline": cls,
        "stages": stages,
        "clocks": clk.summary(),
    }
    if reports(rank) and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_port(vol)
    helper.shutdown()
    ctx_t.close()
    ctx.close()
    rep.close()
    return out if reports(rank) else None


def _sample_slab(vol, z0, nz):
    from tmc_gb300 import volumes
    d = vol.data[z0:z0 + nz].copy()
    return volumes.Volume(d, origin=(vol.origin[0], vol.origin[1], vol.origin[2] + z0 * vol.spacing[2]),
                          spacing=vol.spacing, iso=vol.iso)


def cpu_baseline_port(vol, planes=24):
    """The oracle (a single-threaded C restatement of the reference CPU path) on a bounded sample
    of the same field: a slab of `planes` z-planes, TMC + DMC with simplification."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from cpu_libs import OracleLib
    o = OracleLib()
    s = _sample_slab(vol, 200, planes)
    t0 = time.perf_counter()
    o.tmc(s)
    o.dmc(s, 1)
    dt = time.perf_counter() - t0
    cells = s.cells
    return {"value": round(cells / dt / 1e9, 6), "unit": "Gcells/s", "cores": 1, "kind": "port",
            "sample": f"z-slab of {planes} planes ({s.dims[0]}x{s.dims[1]}x{s.dims[2]}) of the same field, "
                      f"TMC + DMC(simplify), {dt:.2f} s"}


# ------------------------------------------------------------------------------------------------
# reference arm: the reference's own CPU implementation on the host cores
# ------------------------------------------------------------------------------------------------
def _ref_worker(a):
    path, z0, nz, kind = a
    import numpy as np
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from tmc_gb300 import volumes
    import cpu_libs
    data = np.load(path, mmap_mode="r")
    n = data.shape[2]
    d = np.ascontiguousarray(data[z0:z0 + nz])
    vol = volumes.Volume(d, origin=(-1.0, -1.0, -1.0 + z0 * 2.0 / (n - 1)), spacing=(2.0 / (n - 1),) * 3, iso=0.0)
    lib = cpu_libs.RefLib() if kind == "reference" else cpu_libs.OracleLib()
    t0 = time.perf_counter()
    lib.tmc(vol)
    lib.dmc(vol, 1)
    return time.perf_counter() - t0, vol.cells


def run_reference(args, rank, world):
    if rank != 0:
        return None
    import multiprocessing as mp

    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cpu_libs
    from tmc_gb300 import volumes
    kind = "reference" if cpu_libs.ref_available() else "port"
    if kind == "port":
        try:
            cpu_libs.OracleLib()
        except Exception as e:
            return {"impl": "reference", "unavailable": f"oracle could not be built: {e}"}
    vol = volumes.noise_volume(N, seed=SEED)
    path = "/dev/shm/tmc_bench_field.npy" if os.path.isdir("/dev/shm") else os.path.join(ROOT, "_bench_field.npy")
    np.save(path, vol.data)
    cores = os.cpu_count() or 1
    planes = 12
    jobs = [(path, (w * 37) % (N - planes), planes, kind) for w in range(cores)]
    with mp.get_context("spawn").Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_worker, jobs[: max(1, cores // 4)])
        t0 = time.perf_counter()
        cells = 0
        for _ in range(args.steps):
            for dt, c in pool.map(_ref_worker, jobs):
                cells += c
        wall = time.perf_counter() - t0
    try:
        os.remove(path)
    except OSError:
        pass
    value = cells / wall / 1e9
    ms_step = wall / args.steps * 1e3
    return {"impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": "Gcells/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "512^3 noise field, isovalue 0: TMC shared-vertex + DMC with P3X3Y+P3333 "
                                   "simplification, per step one z-slab sample per host core",
                       "grid": [N, N, N], "sample_planes": planes},
            "cpu_baseline": {"value": round(value, 6), "unit": "Gcells/s", "cores": cores, "kind": kind,
                             "sample": f"{cores} slabs of {planes} z-planes of the 512^3 field per step, "
                                       f"one process per core (the CPU path is single-threaded)"},
            "e2e": {"value": round(value, 6), "unit": "Gcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ------------------------------------------------------------------------------------------------
# batch workload: 256 volumes of uneven sizes, DMC shared-vertex quads
# ------------------------------------------------------------------------------------------------
def run_batch(args, rank, world, local):
    import numpy as np
    import torch

    from tmc_gb300 import native, volumes
    try:
        native.load()
    except RuntimeError:
        from tmc_gb300 import build
        build.build()
    torch.cuda.set_device(local)
    vols = volumes.batch_volumes(args.volumes, seed=2 + 1000 * rank)
    cells = sum(v.cells for v in vols)
    voxels = sum(v.data.size for v in vols)
    ctx = native.Context(local)
    devs = [torch.from_numpy(np.ascontiguousarray(v.data)).cuda() for v in vols]
    tv = [native.make_volume(v, d.data_ptr(), on_device=True) for v, d in zip(vols, devs)]
    isos = [v.iso for v in vols]
    n = len(vols)
    stream = torch.cuda.ExternalStream(ctx.stream)

    def batched():
        ms = ctx.batch_raw(tv, isos, [native.ALGO_DMC] * n, [0] * n)
        return ms

    def plain():
        return [ctx.dmc_raw(t, iso, 0) for t, iso in zip(tv, isos)]

    def timed(fn):
        for _ in range(args.warmup):
            for m in fn():
                ctx.free(m)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        total = 0.0
        l0 = ctx.launches()
        for _ in range(args.steps):
            e0.record(stream)
            ms = fn()
            e1.record(stream)
            e1.synchronize()
            total += e0.elapsed_time(e1)
            for m in ms:
                ctx.free(m)
        return total / args.steps, (ctx.launches() - l0) // args.steps, ms

    with ClockSampler(local) as clk:
        ms_batch, launches_batch, _ = timed(batched)
        ms_plain, launches_plain, _ = timed(plain)
    # per-stage device time of one batched call (separate pass, not timed above)
    ctx.set_profiling(True)
    for m in batched():
        ctx.free(m)
    prof = ctx.profile()
    ctx.set_profiling(False)
    batch_stages = {k: round(v[0], 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
    # sizes and the output bytes of one batch
    ms = batched()
    nv = sum(m.nr_v for m in ms)
    nq = sum(m.nr_q for m in ms)
    for m in ms:
        ctx.free(m)
    # end to end: host fields in, host meshes out, through the C ABI
    pins = [torch.from_numpy(np.ascontiguousarray(v.data)).pin_memory() for v in vols]
    th = [native.make_volume(v, p.data_ptr(), on_device=False) for v, p in zip(vols, pins)]
    for m in ctx.batch_raw(th, isos, [native.ALGO_DMC] * n, [native.OUT_HOST] * n):
        ctx.free(m)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for m in ctx.batch_raw(th, isos, [native.ALGO_DMC] * n, [native.OUT_HOST] * n):
            ctx.free(m)
    e2e_s = (time.perf_counter() - t0) / args.steps
    algo_bytes = 4.0 * voxels + 24.0 * nv + 16.0 * nq
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = algo_bytes / (ms_batch * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": round(cells / (ms_batch * 1e-3) / 1e9, 4), "unit": "Gcells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_batch, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n} volumes, each axis log-uniform in [32,192], blob / periodic fields, "
                               "iso U[-0.3,0.3]; DMC shared-vertex quads, one batched call per step",
                   "cells_per_step": cells, "seed": 2, "l2": f"inputs larger than L2 ({4 * voxels / 2**20:.0f} MiB of fields)",
                   "parallelism": f"replicas x{world}"},
        "mesh": {"v": nv, "q": nq},
        "plain_calls": {"value": round(cells / (ms_plain * 1e-3) / 1e9, 4), "unit": "Gcells/s",
                        "ms_per_step": round(ms_plain, 3), "gpu_launches": int(launches_plain),
                        "note": f"{n} sequential tmc_dmc_extract calls"},
        "batched_over_plain": round(ms_plain / ms_batch, 3),
        "stages_ms": batch_stages,
        "e2e": {"value": round(cells / e2e_s / 1e9, 4), "unit": "Gcells/s", "h2d_bytes_per_step": 4 * voxels,
                "d2h_bytes_per_step": int(24 * nv + 16 * nq)},
        "gpu_launches": int(launches_batch),
        "roofline": {"bound": "hbm", "kernel": "whole batch (field read once + mesh written)",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": None, "algorithmic_bytes_per_launch": algo_bytes,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6.8 TB/s"},
        "clocks": clk.summary(),
    }
    ctx.close()
    return out if rank == 0 else None


# ------------------------------------------------------------------------------------------------
# precision stress: 1024^3 periodic field (k = 6 pi) with seeded near-singular saddle faces
# ------------------------------------------------------------------------------------------------
def _position_error(v32, v64, spacing):
    """max and RMS of |float32 position - float64 position| in cell units (per axis spacing)."""
    import numpy as np
    sp = np.asarray(spacing, np.float64)
    mx, ss, cnt = 0.0, 0.0, 0
    step = 3 << 22  # whole vertices per chunk
    for a in range(0, v32.size, step):
        d = np.abs(v32[a:a + step].astype(np.float64) - v64[a:a + step]).reshape(-1, 3) / sp
        mx = max(mx, float(d.max()) if d.size else 0.0)
        ss += float((d * d).sum())
        cnt += d.size
    return {"max": mx, "rms": (ss / cnt) ** 0.5 if cnt else 0.0}


def run_precision(args, rank, world, local):
    import numpy as np
    import torch

    from tmc_gb300 import native, volumes
    try:
        native.load()
    except RuntimeError:
        from tmc_gb300 import build
        build.build()
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from cpu_libs import OracleLib
    oracle = OracleLib()
    torch.cuda.set_device(local)
    n = args.grid if args.grid != N else 1024
    t0 = time.perf_counter()
    vol = volumes.saddle_volume(n, seed=3)
    gen_s = time.perf_counter() - t0
    cells = vol.cells
    ctx = native.Context(local)
    dev = torch.from_numpy(vol.data).cuda()
    v = native.make_volume(vol, dev.data_ptr(), on_device=True)
    stream = torch.cuda.ExternalStream(ctx.stream)

    def step():
        md = ctx.dmc_raw(v, vol.iso, 0)
        mt = ctx.tmc_raw(v, vol.iso, 0)
        return md, mt

    for _ in range(args.warmup):
        for m in step():
            ctx.free(m)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            md, mt = step()
            stats = (list(md.stats), list(mt.stats))
            sizes = {"dmc_v": md.nr_v, "dmc_q": md.nr_q, "tmc_v": mt.nr_v, "tmc_t": mt.nr_t}
            ctx.free(md)
            ctx.free(mt)
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # float32 positions against the float64 ones (bit-equal to the reference's doubles) on the full grid
    mdh = ctx.fetch(ctx.dmc_raw(v, vol.iso, native.OUT_POS_F64 | native.OUT_HOST))
    err_dmc = _position_error(mdh["v"], mdh["v64"], vol.spacing)
    del mdh
    mth = ctx.fetch(ctx.tmc_raw(v, vol.iso, native.OUT_POS_F64 | native.OUT_HOST))
    err_tmc = _position_error(mth["v"], mth["v64"], vol.spacing)
    del mth
    # topology and float64 positions against the oracle on z-slabs of the same field
    planes = 10
    slabs = sorted({0, n // 3, (2 * n) // 3, n - planes})
    mism = {"dmc_quads": 0, "dmc_v64": 0, "tmc_tris": 0, "tmc_v64": 0}
    checked = {"dmc_quads": 0, "tmc_tris": 0}
    t1 = time.perf_counter()
    for z0 in slabs:
        sub = _sample_slab(vol, z0, planes)
        gd = ctx.dmc(sub, native.OUT_POS_F64)
        od = oracle.dmc(sub, 0)
        mism["dmc_quads"] += int(np.count_nonzero(gd["q"] != od["q"])) if gd["q"].shape == od["q"].shape else max(gd["q"].size, od["q"].size)
        mism["dmc_v64"] += int(np.count_nonzero(gd["v64"] != od["v"])) if gd["v64"].shape == od["v"].shape else max(gd["v64"].size, od["v"].size)
        checked["dmc_quads"] += od["q"].size // 4
        gt = ctx.tmc(sub, native.OUT_POS_F64)
        ot = oracle.tmc(sub)
        mism["tmc_tris"] += int(np.count_nonzero(gt["t"] != ot["t"])) if gt["t"].shape == ot["t"].shape else max(gt["t"].size, ot["t"].size)
        mism["tmc_v64"] += int(np.count_nonzero(gt["v64"] != ot["v"])) if gt["v64"].shape == ot["v"].shape else max(gt["v64"].size, ot["v"].size)
        checked["tmc_tris"] += ot["t"].size // 3
    oracle_s = time.perf_counter() - t1
    out = {
        "metric": METRIC, "value": round(cells / (ms * 1e-3) / 1e9, 4), "unit": "Gcells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n}^3 periodic field sin(kx)cos(ky)+sin(ky)cos(kz)+sin(kz)cos(kx), k = 6 pi, with "
                               f"20% of a disjoint face family (xy faces at even i, j) overwritten by bilinear saddles "
                               f"whose decider lies within 1e-6 of the isovalue 0; DMC (no simplification) + TMC per step",
                   "cells_per_step": cells, "seed": 3, "saddle_faces": vol.meta["saddle_faces"],
                   "field_generation_s": round(gen_s, 1), "l2": "inputs larger than L2 (4 GiB field)"},
        "mesh": sizes,
        "float64_fallbacks": {"dmc": stats[0][7], "tmc_singular_faces": stats[1][5]},
        "position_error_cells": {"dmc_float32": err_dmc, "tmc_float32": err_tmc,
                                 "note": "float32 output against the float64 output, which equals the oracle's "
                                         "doubles bit for bit on the checked slabs"},
        "topology_vs_oracle": {"slabs_z0": slabs, "planes_per_slab": planes, "mismatched_entries": mism,
                               "checked": checked, "oracle_seconds": round(oracle_s, 1)},
        "clocks": clk.summary(),
    }
    ctx.close()
    return out if rank == 0 else None


# ------------------------------------------------------------------------------------------------
# serving: Poisson request stream, continuous batching vs one call per request
# ------------------------------------------------------------------------------------------------
def _drive(submit, poll, collect, arrivals):
    """Submit request q at arrivals[q] (seconds from start); a monitor polls every ticket and records
    its completion time.  Returns (latencies in s, makespan in s)."""
    n = len(arrivals)
    tickets = [None] * n
    t_sub = [0.0] * n
    t_done = [None] * n
    start = time.perf_counter()

    def submitter():
        for q in range(n):
            dt = arrivals[q] - (time.perf_counter() - start)
            if dt > 0:
                time.sleep(dt)
            t_sub[q] = time.perf_counter()
            tickets[q] = submit(q)

    th = threading.Thread(target=submitter)
    th.start()
    left = n
    while left:
        for q in range(n):
            if t_done[q] is None and tickets[q] is not None and poll(tickets[q]):
                t_done[q] = time.perf_counter()
                left -= 1
        time.sleep(0.0002)
    th.join()
    for q in range(n):
        collect(tickets[q])
    lat = [t_done[q] - t_sub[q] for q in range(n)]
    return lat, max(t_done) - start


def run_serve(args, rank, world, local):
    import queue

    import numpy as np
    import torch

    from tmc_gb300 import native, volumes
    try:
        native.load()
    except RuntimeError:
        from tmc_gb300 import build
        build.build()
    torch.cuda.set_device(local)
    rng = np.random.Generator(np.random.PCG64(4 + 1000 * rank))
    n = args.requests
    vols = [volumes.serve_request(rng) for _ in range(n)]
    flags = [(0 if q % 2 == 0 else native.OUT_HALFEDGES) | native.OUT_HOST for q in range(n)]
    cells = sum(v.cells for v in vols)
    pins = [torch.from_numpy(np.ascontiguousarray(v.data)).pin_memory() for v in vols]
    tv = [native.make_volume(v, p.data_ptr(), on_device=False) for v, p in zip(vols, pins)]
    ctx = native.Context(local)

    # the plain loop: one thread, one tmc_dmc_extract call per request, in arrival order
    class Plain:
        def __init__(self):
            self.q = queue.Queue()
            self.done = {}
            self.th = threading.Thread(target=self.loop, daemon=True)
            self.th.start()

        def loop(self):
            while True:
                k = self.q.get()
                if k is None:
                    return
                m = ctx.dmc_raw(tv[k], vols[k].iso, flags[k])
                ctx.free(m)
                self.done[k] = True

        def submit(self, k):
            self.q.put(k)
            return k

        def poll(self, k):
            return k in self.done

        def close(self):
            self.q.put(None)
            self.th.join()

    # capacity of the plain loop (closed loop, all requests queued at once)
    pl = Plain()
    lat0, span0 = _drive(pl.submit, pl.poll, lambda k: None, [0.0] * n)
    pl.close()
    capacity = n / span0
    srv = native.Server(local)

    def srv_submit(k):
        return srv.submit(tv[k], vols[k].iso, native.ALGO_DMC, flags[k])

    def srv_collect(t):
        srv.release(srv.wait_raw(t))

    # warm-up: every request once in large batches (the plain loop's capacity run warmed its context
    # the same way), then once at a low arrival rate, where requests run alone: the workers' pinned
    # host blocks are pooled by size class, and a class first seen inside the timed runs would pay
    # for pinning new host memory there
    _drive(srv_submit, srv.poll, srv_collect, [0.0] * n)
    gaps = rng.exponential(1.0 / (0.5 * capacity), size=n)
    _drive(srv_submit, srv.poll, srv_collect, list(np.cumsum(gaps) - gaps[0]))
    results = []
    with ClockSampler(local) as clk:
        for mult in [float(x) for x in args.rates.split(",")]:
            lam = mult * capacity
            gaps = rng.exponential(1.0 / lam, size=n)
            arrivals = list(np.cumsum(gaps) - gaps[0])
            lat_s, span_s = _drive(srv_submit, srv.poll, srv_collect, arrivals)
            pl = Plain()
            lat_p, span_p = _drive(pl.submit, pl.poll, lambda k: None, arrivals)
            pl.close()
            pct = lambda a, p: float(np.percentile(np.asarray(a) * 1e3, p))
            results.append({
                "rate_req_s": round(lam, 2), "rate_over_plain_capacity": mult,
                "server": {"p50_ms": round(pct(lat_s, 50), 2), "p99_ms": round(pct(lat_s, 99), 2),
                           "gcells_s": round(cells / span_s / 1e9, 4)},
                "plain": {"p50_ms": round(pct(lat_p, 50), 2), "p99_ms": round(pct(lat_p, 99), 2),
                          "gcells_s": round(cells / span_p / 1e9, 4)}})
    st = srv.stats()
    srv.close()
    ctx.close()
    best = max(results, key=lambda r: r["server"]["gcells_s"])
    out = {
        "metric": METRIC, "value": best["server"]["gcells_s"], "unit": "Gcells/s", "n_gpus": world,
        "steps": len(results), "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n} requests per rate, per-axis size lognormal (median 128, sigma 0.5) clipped to "
                               "[48, 512], blob / periodic fields, iso U[-0.3, 0.3], DMC shared-vertex or halfedge "
                               "(50/50), host fields in, host meshes out; Poisson arrivals; 120 GB admission budget",
                   "cells_per_rate": cells, "seed": 4, "plain_capacity_req_s": round(capacity, 2)},
        "rates": results,
        "server_stats": {"batches": st[2], "requests": st[3], "largest_batch": st[5], "peak_admitted_bytes": st[4]},
        "e2e": {"value": best["server"]["gcells_s"], "unit": "Gcells/s",
                "h2d_bytes_per_step": int(sum(4 * v.data.size for v in vols)), "d2h_bytes_per_step": None},
        "clocks": clk.summary(),
    }
    return out if rank == 0 else None


# ------------------------------------------------------------------------------------------------
# the 64^3 Gaussian-blob plain DMC call (no simplification), the reference's CPU-runnable case
# ------------------------------------------------------------------------------------------------
def run_plain64(args, rank, world, local):
    import numpy as np
    import torch

    from tmc_gb300 import native, volumes
    try:
        native.load()
    except RuntimeError:
        from tmc_gb300 import build
        build.build()
    torch.cuda.set_device(local)
    vol = volumes.blobs_volume(64, seed=0)
    cells = vol.cells
    ctx = native.Context(local)
    dev = torch.from_numpy(vol.data).cuda()
    vdev = native.make_volume(vol, dev.data_ptr(), on_device=True)
    pin = torch.from_numpy(vol.data).pin_memory()
    vhost = native.make_volume(vol, pin.data_ptr(), on_device=False)
    stream = torch.cuda.ExternalStream(ctx.stream)
    reps = 200  # calls per step: one call is tens of microseconds
    for _ in range(args.warmup * reps):
        ctx.free(ctx.dmc_raw(vdev, vol.iso, 0))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps * reps):
            m = ctx.dmc_raw(vdev, vol.iso, 0)
            nv, nq = m.nr_v, m.nr_q
            ctx.free(m)
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1) / (args.steps * reps)
    t0 = time.perf_counter()
    for _ in range(args.steps * reps):
        ctx.free(ctx.dmc_raw(vhost, vol.iso, native.OUT_HOST))
    e2e_ms = (time.perf_counter() - t0) * 1e3 / (args.steps * reps)
    # per-stage device time of one call (separate pass, not timed above)
    ctx.set_profiling(True)
    for _ in range(20):
        m = ctx.dmc_raw(vdev, vol.iso, 0)
        fails = (m.stats[2], m.stats[3])
        ctx.free(m)
    prof = ctx.profile()
    ctx.set_profiling(False)
    out = {
        "metric": METRIC, "value": round(cells / (ms * 1e-3) / 1e9, 4), "unit": "Gcells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms * reps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "64^3 field of 8 Gaussian blobs on [-1,1]^3 (seed 0), isovalue 0.5: plain DMC "
                               f"(shared-vertex quads, no simplification), {reps} calls per step",
                   "cells_per_call": cells, "ms_per_call": round(ms, 4), "l2": "field resident (1 MiB): latency-bound"},
        "mesh": {"v": nv, "q": nq, "projection_fail_7x7": fails[0], "projection_fail_26x26": fails[1]},
        "stages_us_per_call": {k: round(v[0] / 20 * 1e3, 2) for k, v in prof.items()},
        "e2e": {"value": round(cells / (e2e_ms * 1e-3) / 1e9, 4), "unit": "Gcells/s", "ms_per_call": round(e2e_ms, 4),
                "h2d_bytes_per_step": 4 * vol.data.size * reps, "d2h_bytes_per_step": (24 * nv + 16 * nq) * reps},
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from cpu_libs import OracleLib
        o = OracleLib()
        t0 = time.perf_counter()
        for _ in range(5):
            o.dmc(vol, 0)
        dt = (time.perf_counter() - t0) / 5
        out["cpu_baseline"] = {"value": round(cells / dt / 1e9, 6), "unit": "Gcells/s", "cores": 1, "kind": "port",
                               "sample": f"the whole 64^3 field, plain DMC, {dt * 1e3:.1f} ms per call"}
    ctx.close()
    return out if rank == 0 else None


# ------------------------------------------------------------------------------------------------
# fused generation: the field evaluated inside the classification instead of generated and read
# ------------------------------------------------------------------------------------------------
def run_fused(args, rank, world, local, steps=None, warmup=None):
    """Generated 512^3 fields (the periodic field with k = 6 pi, isovalue 0, and the reference's sphere):
    per step one DMC (shared-vertex quads) and one TMC (shared-vertex triangles) extraction, either
    stored (tmc_field_generate_ex writes the field, then the extractions read it) or fused
    (tmc_*_extract_generated: the classification evaluates the field).  The fused classification's
    ALU roofline is its rate of field evaluations against the rate of the standalone generation
    kernel, which does nothing but evaluate and store (one evaluation per point)."""
    import torch

    from tmc_gb300 import native
    try:
        native.load()
    except RuntimeError:
        from tmc_gb300 import build
        build.build()
    torch.cuda.set_device(local)
    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup
    n = args.grid
    ctx = native.Context(local)
    cells = (n - 1) ** 3
    gens = {"periodic_k6pi": (native.make_generator(native.SURF_PERIODIC, (n, n, n), (6 * math.pi,)), 0.0),
            "sphere": (native.make_generator(0, (n, n, n)), 0.0)}
    results = {}
    for name, (gen, iso) in gens.items():
        def stored():
            f = ctx.field_generate_ex(gen)
            ctx.free(ctx.dmc_raw(f.vol, iso, 0))
            ctx.free(ctx.tmc_raw(f.vol, iso, 0))
            ctx.field_free(f)

        def fused():
            ctx.free(ctx.dmc_generated_raw(gen, iso, 0))
            ctx.free(ctx.tmc_generated_raw(gen, iso, 0))

        def generate_only():
            ctx.field_free(ctx.field_generate_ex(gen))

        def timed(fn, k):
            for _ in range(warmup):
                fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(k):
                fn()
            ctx.synchronize()
            return (time.perf_counter() - t0) / k * 1e3

        with ClockSampler(local) as clk:
            ms_stored = timed(stored, steps)
            ms_fused = timed(fused, steps)
            ms_gen = timed(generate_only, steps)
        # the fused classification alone (stage timing on the context stream)
        ctx.set_profiling(True)
        ctx.free(ctx.dmc_generated_raw(gen, iso, 0))
        ctx.free(ctx.tmc_generated_raw(gen, iso, 0))
        prof = ctx.profile()
        ctx.set_profiling(False)
        # evaluations of the fused classification: four corner rows per cell, four more on the lanes
        # that load their x+1 points themselves (a warp's last lane and a row's last cell)
        evals = 4 * cells * (1 + 1 / 32 + 1 / (n - 1))
        gen_rate = n ** 3 / (ms_gen * 1e-3)
        cls = {}
        for st in ("dmc_classify", "tmc_classify"):
            if st in prof:
                ms = prof[st][0] / max(prof[st][1], 1)
                rate = evals / (ms * 1e-3)
                cls[st] = {"ms": round(ms, 4), "evals_per_s": round(rate / 1e9, 2),
                           "frac_of_generation_rate": round(rate / gen_rate, 3)}
        results[name] = {
            "stored_ms_per_step": round(ms_stored, 3), "fused_ms_per_step": round(ms_fused, 3),
            "stored_gcells_s": round(cells / (ms_stored * 1e-3) / 1e9, 4),
            "fused_gcells_s": round(cells / (ms_fused * 1e-3) / 1e9, 4),
            "fused_over_stored": round(ms_stored / ms_fused, 3),
            "generation_call_ms": round(ms_gen, 3), "generation_gevals_s": round(gen_rate / 1e9, 2),
            "fused_classify": cls, "clocks": clk.summary()}
    ctx.close()
    return {"workload": f"generated {n}^3 fields, isovalue 0: DMC shared-vertex + TMC shared-vertex per step; "
                        "stored = generate the field then extract, fused = the classification evaluates the field",
            "steps": steps, "warmup": warmup, "fields": results,
            "roofline": "ALU: the fused classification's field evaluations per second against the generation "
                        "kernel's (one evaluation and one 4-byte store per point; for the periodic field its "
                        "six float32 sin/cos bound it, for the sphere the store)",
            "note": "timed on the host clock with a synchronisation per step (the stored path allocates and frees "
                    "its field each step)"}


def headline_extras(args, rank, world, local):
    """The batched and served workloads, measured beside the default one so that one bench line
    carries the whole headline metric: `batch` (256 uneven volumes in one batched call against 256
    plain calls) and `serve` (Poisson arrivals at two rates, the server against one call per request)."""
    if world > 1:
        note = "measured at one GPU only (each replica would run the same independent workload)"
        return {"batch": {"note": note}, "serve": {"note": note}}
    extras = {}
    bargs = argparse.Namespace(**vars(args))
    bargs.steps, bargs.warmup, bargs.volumes = 3, 3, 256
    b = run_batch(bargs, rank, world, local)
    extras["batch"] = {
        "value": b["value"], "unit": "Gcells/s", "ms_per_batch": b["ms_per_step"], "volumes": bargs.volumes,
        "cells_per_batch": b["config"]["cells_per_step"], "gpu_launches_per_batch": b["gpu_launches"],
        "plain_calls": {"value": b["plain_calls"]["value"], "ms": b["plain_calls"]["ms_per_step"],
                        "gpu_launches": b["plain_calls"]["gpu_launches"]},
        "batched_over_plain": b["batched_over_plain"], "e2e": b["e2e"], "stages_ms": b["stages_ms"],
        "roofline": {k: b["roofline"][k] for k in ("achieved", "peak", "unit", "frac", "algorithmic_bytes_per_launch")},
        "workload": b["config"]["workload"], "steps": bargs.steps, "warmup": bargs.warmup, "clocks": b["clocks"]}
    sargs = argparse.Namespace(**vars(args))
    sargs.requests, sargs.rates = 256, "0.5,1.5"
    import torch
    link = link_bandwidth(torch)
    sv = run_serve(sargs, rank, world, local)
    fargs = argparse.Namespace(**vars(args))
    extras["fused_generation"] = run_fused(fargs, rank, world, local, steps=5, warmup=3)
    extras["serve"] = {"rates": sv["rates"], "plain_capacity_req_s": sv["config"]["plain_capacity_req_s"],
                       "requests_per_rate": sargs.requests, "workload": sv["config"]["workload"],
                       "server_stats": sv["server_stats"], "clocks": sv["clocks"],
                       "host_link_gbs": link,
                       "note": "every request's field crosses the host link in and its mesh out, on both arms; the link "
                               "is shared with the machine's other GPUs, so both arms' latencies vary between runs"}
    return extras


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload == "single" and args.grid == N and not args.no_extras:
        out = run_ours(args, rank, world, local)
        extra = headline_extras(args, rank, world, local)
        if out is not None:
            out.update(extra)
    elif args.workload == "batch":
        out = run_batch(args, rank, world, local)
    elif args.workload == "precision":
        out = run_precision(args, rank, world, local)
    elif args.workload == "serve":
        out = run_serve(args, rank, world, local)
    elif args.workload == "plain64":
        out = run_plain64(args, rank, world, local)
    elif args.workload == "fused":
        out = run_fused(args, rank, world, local)
    else:
        out = run_ours(args, rank, world, local)
    if out is not None and rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
