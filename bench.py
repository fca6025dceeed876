#!/usr/bin/env python
"""Voxel-queries/s of the GB300 voxelization path (occupancy + signed distance).

Workload: the star-shaped spherical-harmonic surface of 65,024 triangles (UV
sphere, 256 x 128 bands, radius 1 + 8 real harmonics of degree <= 6, seed 3),
voxelized with 256 cells on its longest axis (resolution 254, pad 1). One step =
occupancy (exact ray parity, reference predicates) + the mixed-precision signed
distance field (FP32 on brick-recentred coordinates, FP64 within one cell of the
surface) for every cell; a voxel query = one cell's occupancy bit + SDF value.
The plain all-FP64 path (bit-identical to the reference) is timed beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload sdf|batch|scale|stream|stl|detect]

The default workload (sdf) is the headline above. The others measure the rest of
the path, each printing one line of the same form:
  batch   512 meshes (icospheres / tori, resolutions 32-192) in one pipeline,
          occupancy + mixed SDF, replayed as a CUDA graph, autotuned;
  scale   2000 ellipsoids (2.56M triangles) at 512^3: forward (occupancy + mixed
          SDF + nearest-feature checkpoint) and the adjoint per step;
  stream  1e8 orient3d + 1e8 insphere sign queries (10 % exactly degenerate),
          reference semantics;
  stl     a binary STL image of the 2000 ellipsoids (2.56M triangles) read into a PLC
          (records decoded, coincident vertices merged);
  detect  the self-intersection preflight of the same 2.56M triangles.

Under torchrun each rank runs its own replica (weak scaling; the path shares
nothing between meshes), the timed region is bracketed by barriers and the
slowest rank's time is used. --impl reference times the CPU restatement of the
reference algorithm (oracle/, the reference's own code cannot travel to the GPU
host) on this host's cores, on bounded samples of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "voxel-queries/s, 256³ grid/65k tris: mixed vs FP64 GPU at SDF err≤1e-6·diag"
UNIT = "voxel-queries/s"
RESOLUTION, PAD = 254, 1
PT_FLOPS = 79      # FP64 flops of one Ericson point-triangle evaluation (interior path)
O3D_FLOPS = 23     # flops of one rounded orient3d determinant
PZ_FLOPS = 22      # flops of one plane_z
L2_FLUSH_BYTES = 256 << 20


PINNED_MESH = os.path.join(ROOT, "tests", "golden", "shsphere256.npz")


def workload():
    """The headline mesh as serialised float64 bits (the input the full-size parity
    tests check against the reference's outputs), else regenerated."""
    if os.path.exists(PINNED_MESH):
        with np.load(PINNED_MESH) as z:
            return np.array(z["points"]), np.array(z["triangles"])
    from cybermeshgenerator_gb300 import workloads as W
    return W.sh_sphere(nlon=256, nlat=128, seed=3)


def kernel_source_sha(files=("sdf_sub.cu", "cmg_sdf.cuh")):
    """SHA-256 (16 hex digits) of the evaluation kernel's code (the sources with their
    // comments and blank lines taken out), recorded in its ncu summary so that the bench
    line takes DRAM traffic only from a capture of this code."""
    import hashlib
    h = hashlib.sha256()
    for f in files:
        with open(os.path.join(ROOT, "cybermeshgenerator_gb300", "csrc", f), encoding="utf-8") as fh:
            for line in fh:
                code = line.split("//", 1)[0].rstrip()
                if code:
                    h.update(code.encode() + b"\n")
    return h.hexdigest()[:16]


def workload_desc(dims, ntris):
    return {"workload": f"SH star surface, {ntris} triangles, resolution {RESOLUTION} pad {PAD} "
                        f"({dims[0]}x{dims[1]}x{dims[2]} cells): occupancy + mixed SDF",
            "triangles": int(ntris), "grid": [int(d) for d in dims],
            "precision": "FP32 SDF on brick-recentred coordinates, FP64 band of 1 cell, FP64 predicates",
            "l2": "flushed between timed steps (256 MB device write on the same stream)"}


# --------------------------------------------------------------------------- dist
def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi sampling during the timed region (SM clock + throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.f = None

    def __enter__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.f.name) as fh:
                for line in fh:
                    p = [x.strip() for x in line.split(",")]
                    if len(p) >= 9 and p[1].isdigit():
                        rows.append(p)
            os.unlink(self.f.name)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [int(r[1]) for r in rows]
        mx = int(rows[0][2])
        loaded = [s for s, r in zip(sm, rows) if float(r[3] or 0) > 200.0] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v == "Active"})
        return {"sm_mhz": float(statistics.median(loaded)), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


# --------------------------------------------------------------------------- ours
def time_batch(cm, torch, batch, steps, warmup, flush):
    """Device time of `steps` passes (CUDA events on the batch's stream), L2
    flushed between passes outside the timed events."""
    stream = torch.cuda.ExternalStream(batch.stream)
    for _ in range(warmup):
        batch.run()
    batch.sync()
    times = []
    with torch.cuda.stream(stream):
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            batch.run()
            e1.record(stream)
            times.append((e0, e1))
    batch.sync()
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in times]


def fraction_of_peak(work_flops, ms, peak):
    achieved = work_flops / (ms * 1e-3)
    return achieved, achieved / peak


TRAFFIC_PROFILE = os.path.join("profiles", "k_sdf_sub_mixed_shsphere256.md")


def traffic_from_profile():
    """DRAM bytes per launch of the evaluation kernel from the committed ncu summary,
    when that capture was of the current kernel source: (bytes or None, note)."""
    path = os.path.join(ROOT, TRAFFIC_PROFILE)
    vals = {}
    try:
        with open(path) as f:
            for line in f:
                for key in ("dram_bytes_per_launch:", "kernel_source_sha:"):
                    if line.startswith(key):
                        vals[key] = line.split(":", 1)[1].split()[0]
    except OSError:
        return None, "no ncu summary"
    sha = kernel_source_sha()
    if vals.get("kernel_source_sha:") != sha:
        return None, f"{TRAFFIC_PROFILE} was captured from other kernel sources (now {sha})"
    return float(vals["dram_bytes_per_launch:"]), f"{TRAFFIC_PROFILE}, ncu capture of kernel sources {sha}"


def stream_traffic_per_query():
    """DRAM bytes per query of the FP32 stream passes (orient3d, insphere) from the
    committed ncu summary, when that capture was of the current predicates.cu."""
    path = os.path.join(ROOT, "profiles", "k_pred_fp32_tma_stream2e7.md")
    q, sha = None, None
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("dram_bytes_per_query:"):
                    w = line.split(":", 1)[1].split()
                    q = float(w[w.index("orient3d") + 1]), float(w[w.index("insphere") + 1])
                elif line.startswith("kernel_source_sha:"):
                    sha = line.split(":", 1)[1].split()[0]
    except (OSError, ValueError, IndexError):
        return None
    return q if sha == kernel_source_sha(("predicates.cu",)) else None


def cpu_baseline(pts, tris, dims_grid, seconds=12.0, threads=None, probe=2000):
    """The oracle (CPU restatement of the reference algorithm) on this host: full
    occupancy plus the ring-search SDF on a uniform sample of cells, scaled to
    the grid. threads=None: every host core."""
    import oracle
    orc = oracle.Oracle()
    threads = threads or os.cpu_count() or 1
    corner, spacing, dims = dims_grid
    g = orc.grid(corner, spacing, dims)
    n = g.ncell
    t0 = time.perf_counter()
    orc.occupancy(pts, tris, g, threads=threads)
    t_occ = time.perf_counter() - t0
    rng = np.random.default_rng(7)
    # size the sample from a small probe so the run stays near `seconds`; the
    # oracle times its bucket build and its queries separately
    pv = rng.choice(n, size=min(n, probe), replace=False)
    _, (t_build, t_q) = orc.sdf_ring_sample(pts, tris, g, pv, threads=threads, times=True)
    per = max(t_q / len(pv), 1e-9)
    m = int(min(n, max(probe, (seconds - t_occ - 2 * t_build) / per)))
    vox = rng.choice(n, size=m, replace=False)
    _, (t_build, t_q) = orc.sdf_ring_sample(pts, tris, g, vox, threads=threads, times=True)
    t_full = t_occ + t_build + t_q / m * n
    return {"value": n / t_full, "unit": UNIT, "cores": int(threads), "kind": "port",
            "sample": f"occupancy on all {n} cells; ring-search SDF on {m} uniformly sampled cells "
                      f"({100.0 * m / n:.3g} % of the grid) + the 3-D bucket build, scaled to {n} "
                      f"cells (extrapolated)",
            "sample_fraction": m / n, "seconds": time.perf_counter() - t0}


def cpu_baselines(pts, tris, dims_grid, seconds):
    """The single-threaded figure (the reference voxelizer runs on one thread), with
    the all-cores figure of the same port beside it."""
    one = cpu_baseline(pts, tris, dims_grid, seconds=seconds, threads=1, probe=300)
    allc = cpu_baseline(pts, tris, dims_grid, seconds=seconds)
    one["all_cores"] = {k: allc[k] for k in ("value", "cores", "sample", "sample_fraction")}
    return one


def tunables(args):
    """Options of the SDF pipeline: the library's autotuner (brick edge, queue grab,
    walk warps, probe head, evaluation CTAs per SM, timed on this input) unless a
    brick edge or a tunable is given on the command line or --no-autotune is set."""
    fixed = {k: v for k, v in (("brick", args.brick), ("walk_warps", args.walk_warps),
                                ("probe", args.probe), ("ctas", args.ctas)) if v}
    return dict(fixed, autotune=not fixed and not args.no_autotune)


def chosen(stats):
    return {k: int(stats[k]) for k in ("brick", "grab", "walk_warps", "probe", "ctas")}


def run_ours(args):
    import torch
    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import build as B
    if rank == 0 or world == 1:
        B.build()
    barrier(world)
    pts, tris = workload()
    plc = cm.PLC.from_arrays(pts, tris)
    outs = cm.OUT_OCCUPANCY | cm.OUT_SDF_F32
    tune = tunables(args)
    mixed = cm.Batch([plc], [RESOLUTION], [PAD], outputs=outs, precision=cm.PREC_MIXED, band=1.0,
                     stage=args.stage, **tune)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    mixed.run().sync()  # sizing pass
    cells = mixed.cells
    r0 = mixed.result(0)
    dims = r0.dims

    l0 = cm.gpu_launches()
    barrier(world)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        ms = time_batch(cm, torch, mixed, args.steps, args.warmup, flush)
    barrier(world)
    launches = (cm.gpu_launches() - l0) // (args.steps + args.warmup)
    total_ms = max_over_ranks(sum(ms), world)
    value = cells * world * args.steps / (total_ms * 1e-3)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64", "data": "synthetic",
            "config": dict(workload_desc(dims, len(tris)), parallelism=f"replicas x{world}"),
            "gpu_launches": int(launches)}
    line["config"]["mesh"] = "serialised float64 bits (tests/golden/shsphere256.npz)" \
        if os.path.exists(PINNED_MESH) else "regenerated"
    clocks = clk.summary()
    line["clocks"] = clocks

    if rank == 0:
        # phase times + cost model (one timed pass of each path)
        mixed.set_timing(True)
        mixed.run().sync()
        tm = mixed.timing()
        wm = mixed.work_model()
        st = mixed.stats()
        line["config"]["tuning"] = dict(chosen(st), autotuned=bool(tune["autotune"]))
        # every candidate evaluated in FP64 (the reference's arithmetic throughout)
        plain = cm.Batch([plc], [RESOLUTION], [PAD], outputs=outs, precision=cm.PREC_FP64_PLAIN, **tune)
        plain.run().sync()
        p_ms = time_batch(cm, torch, plain, max(1, min(3, args.steps)), 1, flush)
        plain.set_timing(True)
        plain.run().sync()
        tp = plain.timing()
        p_value = cells * len(p_ms) / (sum(p_ms) * 1e-3)
        # the library's FP64 path (the FP32 pass, then the FP64 distance of each cell's
        # near-ties): the same bits as the plain one, checked here on the whole grid
        exact = cm.Batch([plc], [RESOLUTION], [PAD], outputs=outs, precision=cm.PREC_FP64, **tune)
        exact.run().sync()
        x_ms = time_batch(cm, torch, exact, max(3, args.steps), 1, flush)
        exact.set_timing(True)
        exact.run().sync()
        tx, sx = exact.timing(), exact.stats()
        x_e2e = []
        for i in range(4):
            t0 = time.perf_counter()
            cm.voxelize_ex(plc, resolution=RESOLUTION, pad=PAD, outputs=outs, precision=cm.PREC_FP64,
                           **tune)
            if i >= 1:
                x_e2e.append(time.perf_counter() - t0)
        # accuracy of this run: mixed vs plain (FP64, bit-identical to the reference)
        rm, rp = mixed.result(0), plain.result(0)
        rx = exact.result(0)
        line["fp64_exact"] = {
            "value": cells * len(x_ms) / (sum(x_ms) * 1e-3),
            "e2e": cells / (sum(x_e2e) / len(x_e2e)),
            "identical_to_plain": bool(np.array_equal(rx.occupancy, rp.occupancy) and
                                       np.array_equal(rx.sdf32.view(np.uint32), rp.sdf32.view(np.uint32))),
            "eval_ms": tx["eval_ms"], "phase_ms": tx, "plain_eval_ms": tp["eval_ms"],
            "evaluations": int(sx["evaluations"]), "fp64_evaluations": int(sx["fp64_evaluations"]),
            "band_cells": int(sx["band_cells"]), "tuning": chosen(sx),
            "path": "CMG_PREC_FP64 (the default of cmg_plc_voxelize): FP32 pass with bounds "
                    "widened to every near-tie of the FP32 minimum, FP64 distances in the "
                    "reference's order over those; plain = CMG_PREC_FP64_PLAIN"}
        diag = float(np.linalg.norm(pts.max(0) - pts.min(0)))
        err = np.abs(rm.sdf32.astype(np.float64) - rp.sdf32.astype(np.float64))
        occ_same = bool(np.array_equal(rm.occupancy, rp.occupancy))
        p32 = cm.peak_flops(False)
        p64 = cm.peak_flops(True)
        w_sdf = wm["sum_k"] * PT_FLOPS
        ach, frac = fraction_of_peak(w_sdf, tm["eval_ms"], p32)
        ach64, frac64 = fraction_of_peak(w_sdf, tp["eval_ms"], p64)
        traffic, traffic_note = traffic_from_profile()
        line["roofline"] = {
            "bound": "fp32", "kernel": "k_sdf_sub<mixed> (distance evaluation)",
            "achieved": ach / 1e12, "peak": p32 / 1e12, "unit": "TFLOP/s", "frac": frac,
            "traffic": traffic, "traffic_source": traffic_note,
            "work": f"sum_v K(v) * {PT_FLOPS} = {w_sdf:.4g} flops per launch; K(v) = triangles whose "
                    f"bounding sphere reaches the cell's distance sphere",
            "peak_source": "measured FFMA microbenchmark on this GPU (no FP32 entry in MEASURED_PEAKS.json)",
            "eval_ms": tm["eval_ms"], "phase_ms": tm,
            "fp64_kernel": {"kernel": "k_sdf_sub<fp64>", "achieved": ach64 / 1e12, "peak": p64 / 1e12,
                            "frac": frac64, "eval_ms": tp["eval_ms"], "phase_ms": tp,
                            "tuning": chosen(plain.stats()),
                            "peak_source": "measured DFMA microbenchmark (FMA = 2 flops)"}}
        line["mixed_vs_fp64"] = {"fp64_value": p_value, "speedup": value / world / p_value,
                                 "max_abs_err": float(err.max()), "rms_err": float(np.sqrt((err ** 2).mean())),
                                 "tol": 1e-6 * diag, "within_tol": bool(err.max() <= 1e-6 * diag),
                                 "occupancy_identical": occ_same,
                                 "band_cells": int(st["band_cells"]),
                                 "evaluations": int(st["evaluations"]),
                                 "fp64_evaluations": int(st["fp64_evaluations"]),
                                 "candidates": int(st["candidates"]),
                                 "subbrick_entries": int(st["filtered"])}
        # end to end through the C ABI with host buffers (upload, pipeline, download)
        e2e_t = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            r = cm.voxelize_ex(plc, resolution=RESOLUTION, pad=PAD, outputs=outs,
                               precision=cm.PREC_MIXED, band=1.0, stage=args.stage, **tune)
            if i >= args.warmup:
                e2e_t.append(time.perf_counter() - t0)
        line["e2e"] = {"value": cells / (sum(e2e_t) / len(e2e_t)), "unit": UNIT,
                       "h2d_bytes_per_step": int(pts.nbytes + tris.nbytes),
                       "d2h_bytes_per_step": int(cells * (1 + 4)),
                       "call": "cmg_plc_voxelize_ex (mixed, occupancy + float SDF), host buffers"}
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baselines(pts, tris, (r0.corner, r0.spacing, r0.dims),
                                                 seconds=args.cpu_seconds)
        print(json.dumps(line), flush=True)
    barrier(world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# --------------------------------------------------------------------------- reference
def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    oracle.build()
    from cybermeshgenerator_gb300 import workloads as W  # noqa: F401
    pts, tris = workload()
    orc = oracle.Oracle()
    g = orc.make_grid(pts, RESOLUTION, PAD)
    budget = max(5.0, min(20.0, 150.0 / max(1, args.steps + args.warmup)))
    vals = []
    base = None
    for i in range(args.warmup + args.steps):
        base = cpu_baseline(pts, tris, (tuple(g.corner), g.spacing, g.dims), seconds=budget)
        if i >= args.warmup:
            vals.append(base["value"])
    value = float(statistics.median(vals))
    base["value"] = value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": g.ncell / value * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
            "config": dict(workload_desc(g.dims, len(tris)), parallelism=f"replicas x{world}",
                           mesh="serialised float64 bits (tests/golden/shsphere256.npz)"
                           if os.path.exists(PINNED_MESH) else "regenerated"),
            "cpu_baseline": base,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)

# --------------------------------------------------------------------------- other workloads
def _base_line(metric, unit, value, world, args, total_ms, dtype, config, launches, clocks,
               higher=True):
    return {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": higher, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic", "config": config, "gpu_launches": int(launches),
            "clocks": clocks}


def _events_time(torch, stream, fn, steps, warmup, flush=None):
    """Device time of `steps` calls of fn() (CUDA events on `stream`)."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    pairs = []
    with torch.cuda.stream(stream):
        for _ in range(steps):
            if flush is not None:
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            pairs.append((e0, e1))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in pairs]


BATCH_METRIC = "voxel-queries/s, batch of 512 meshes (80-131k tris, 32^3-192^3): occupancy + mixed SDF"
SCALE_METRIC = "voxel-queries/s, 512^3 grid/2.56M tris: occupancy + mixed SDF + adjoint"
STREAM_METRIC = "predicate queries/s, 1e8 orient3d + 1e8 insphere (10% degenerate), reference semantics"
STREAM_NEAR = 0.1  # the harder mix reported beside: another 10 % within a few ulps of a tie


def _batch_workload():
    from cybermeshgenerator_gb300 import workloads as W
    return W.mesh_batch(512)


def run_batch(args):
    import torch
    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import build as B
    if rank == 0 or world == 1:
        B.build()
    barrier(world)
    items = _batch_workload()
    plcs = [cm.PLC.from_arrays(b.points, b.triangles) for b in items]
    res, pads = [b.resolution for b in items], [b.pad for b in items]
    outs = cm.OUT_OCCUPANCY | cm.OUT_SDF_F32
    bt = cm.Batch(plcs, res, pads, outputs=outs, precision=cm.PREC_MIXED, autotune=True)
    bt.run(graph=True).sync()  # sizing
    bt.run(graph=True).sync()  # capture + replay
    cells = bt.cells
    stream = torch.cuda.ExternalStream(bt.stream)
    l0 = cm.gpu_launches()
    barrier(world)
    with Clocks(local) as clk:
        ms = _events_time(torch, stream, lambda: bt.run(graph=True), args.steps, args.warmup)
    barrier(world)
    # graph replays launch kernels the host counter does not see: count one eager pass
    e0 = cm.gpu_launches()
    bt.run().sync()
    launches = cm.gpu_launches() - e0
    total_ms = max_over_ranks(sum(ms), world)
    value = cells * world * args.steps / (total_ms * 1e-3)
    ntris = sum(len(b.triangles) for b in items)
    st = bt.stats()
    config = {"workload": f"batch of {len(items)} meshes (icosphere subdivision 1-5 / torus 16-256 "
                          f"segments, scale 0.5-2, random rotation), {ntris} triangles, "
                          f"resolutions 32-192 pad 1, {cells} cells: occupancy + mixed SDF",
              "meshes": len(items), "triangles": int(ntris), "cells": int(cells),
              "autotuned": chosen(st),
              "replay": "CUDA graph", "l2": "inputs and outputs larger than L2",
              "parallelism": f"replicas x{world}"}
    line = _base_line(BATCH_METRIC, UNIT, value, world, args, total_ms, "fp32+fp64", config,
                      launches, clk.summary())
    if rank == 0:
        bt.set_timing(True)
        bt.run().sync()
        tm = bt.timing()
        wm = bt.work_model()
        line["config"]["autotuned"] = chosen(bt.stats())
        p32 = cm.peak_flops(False)
        w_sdf = wm["sum_k"] * PT_FLOPS
        ach, frac = fraction_of_peak(w_sdf, tm["eval_ms"], p32)
        line["roofline"] = {"bound": "fp32", "kernel": "k_sdf_sub<mixed> (distance evaluation)",
                            "achieved": ach / 1e12, "peak": p32 / 1e12, "unit": "TFLOP/s",
                            "frac": frac, "traffic": None, "eval_ms": tm["eval_ms"], "phase_ms": tm,
                            "work": f"sum_v K(v) * {PT_FLOPS} = {w_sdf:.4g} flops per launch",
                            "peak_source": "measured FFMA microbenchmark on this GPU"}
        # end to end: one public batch call per step (plan + upload, pass, download)
        e2e_t = []
        for i in range(1 + min(args.steps, 3)):
            t0 = time.perf_counter()
            b2 = cm.Batch(plcs, res, pads, outputs=outs, precision=cm.PREC_MIXED, autotune=True)
            b2.run().sync()
            for k in range(len(items)):
                b2.result(k)
            del b2
            if i:
                e2e_t.append(time.perf_counter() - t0)
        line["e2e"] = {"value": cells / (sum(e2e_t) / len(e2e_t)), "unit": UNIT,
                       "h2d_bytes_per_step": int(sum(b.points.nbytes + b.triangles.nbytes for b in items)),
                       "d2h_bytes_per_step": int(cells * 5),
                       "call": "cmg_batch_create + cmg_batch_run + cmg_batch_get for every mesh"}
        if not args.no_cpu:
            line["cpu_baseline"] = _batch_cpu(items, args.cpu_seconds)
        print(json.dumps(line), flush=True)
    barrier(world)


def _batch_cpu(items, seconds, threads=None):
    """The oracle on every 64th mesh (occupancy + sampled ring SDF, extrapolated per
    mesh), summed: voxel-queries/s of the whole batch at that rate."""
    import oracle
    orc = oracle.Oracle()
    tot_cells, tot_t = 0, 0.0
    sel = items[::64]
    for b in sel:
        g = orc.make_grid(b.points, b.resolution, b.pad)
        r = cpu_baseline(b.points, b.triangles, (tuple(g.corner), g.spacing, g.dims),
                         seconds=max(1.0, seconds / len(sel)), threads=threads)
        tot_cells += g.ncell
        tot_t += g.ncell / r["value"]
    return {"value": tot_cells / tot_t, "unit": UNIT, "cores": int(threads or os.cpu_count() or 1),
            "kind": "port", "sample": f"{len(sel)} of the {len(items)} meshes (every 64th): full "
            "occupancy + ring-search SDF on sampled cells, extrapolated per mesh"}


def _scale_workload():
    from cybermeshgenerator_gb300 import workloads as W
    return W.ellipsoid_field()


def run_scale(args):
    import torch
    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import build as B
    if rank == 0 or world == 1:
        B.build()
    barrier(world)
    import oracle
    from cybermeshgenerator_gb300 import torch_sdf as TS
    pts, tris = _scale_workload()
    g = oracle.Oracle().make_grid(pts, 510, 1)
    grid = TS.grid_of(list(g.corner), g.spacing, (g.nx, g.ny, g.nz))
    plan = TS.SDFPlan(pts, tris, grid, precision=cm.PREC_MIXED, autotune=True)
    v = torch.tensor(pts, device="cuda")
    sdf, occ, tri, reg = plan.forward(v)  # sizing
    rng = np.random.default_rng(53)
    w = torch.tensor(rng.uniform(0.0, 1.0, g.ncell), device="cuda")
    t = torch.tensor(rng.normal(0.0, 0.01, g.ncell), device="cuda")
    state = {}

    def step():
        s_, o_, t_, r_ = plan.forward(None)
        gs = 2.0 * w * (s_ - t)
        state["grad"] = plan.backward(v, o_, t_, r_, gs)

    stream = torch.cuda.current_stream()
    l0 = cm.gpu_launches()
    barrier(world)
    with Clocks(local) as clk:
        ms = _events_time(torch, stream, step, args.steps, args.warmup)
    barrier(world)
    launches = (cm.gpu_launches() - l0) // (args.steps + args.warmup)
    total_ms = max_over_ranks(sum(ms), world)
    cells = g.ncell
    value = cells * world * args.steps / (total_ms * 1e-3)
    config = {"workload": f"2000 ellipsoids (semi-axes U(0.01,0.04), icosphere subdivision 3), "
                          f"{len(tris)} triangles, resolution 510 pad 1 ({g.nx}x{g.ny}x{g.nz} cells): "
                          "occupancy + mixed SDF + nearest-feature checkpoint, then the adjoint of "
                          "sum w (sdf - t)^2",
              "triangles": int(len(tris)), "grid": [g.nx, g.ny, g.nz],
              "l2": "inputs and outputs larger than L2", "parallelism": f"replicas x{world}"}
    line = _base_line(SCALE_METRIC, UNIT, value, world, args, total_ms, "fp32+fp64", config,
                      launches, clk.summary())
    if rank == 0:
        fwd = _events_time(torch, stream, lambda: plan.forward(None), 2, 1)
        s_, o_, t_, r_ = plan.forward(None)
        gs = 2.0 * w * (s_ - t)
        bwd = _events_time(torch, stream, lambda: plan.backward(v, o_, t_, r_, gs), 3, 1)
        # algorithmic bytes of one adjoint: the checkpoint (triangle 4 B, region 1 B,
        # occupancy 1 B) and dL/dsdf (8 B) per cell, the points read and the gradient
        # written (24 B each per point), the triangles (12 B each)
        adj_bytes = cells * (4 + 1 + 1 + 8) + len(pts) * 48 + len(tris) * 12
        hbm = _measured_hbm()
        line["phases_ms"] = {"forward": sum(fwd) / len(fwd), "adjoint": sum(bwd) / len(bwd)}
        # the dominant kernel of the step is the forward's evaluation: its cost model
        # on a batch over the same grid (phase timing and K(v) counting pass)
        bt = cm.Batch([cm.PLC.from_arrays(pts, tris)], outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F32,
                      precision=cm.PREC_MIXED, grid=grid, autotune=True)
        bt.run().sync()
        bt.set_timing(True)
        bt.run().sync()
        tm = bt.timing()
        wm = bt.work_model()
        line["config"]["autotuned"] = chosen(bt.stats())
        p32 = cm.peak_flops(False)
        w_sdf = wm["sum_k"] * PT_FLOPS
        ach, frac = fraction_of_peak(w_sdf, tm["eval_ms"], p32)
        line["roofline"] = {"bound": "fp32", "kernel": "k_sdf_sub<mixed> (distance evaluation)",
                            "achieved": ach / 1e12, "peak": p32 / 1e12, "unit": "TFLOP/s",
                            "frac": frac, "traffic": None, "eval_ms": tm["eval_ms"], "phase_ms": tm,
                            "work": f"sum_v K(v) * {PT_FLOPS} = {w_sdf:.4g} flops per launch",
                            "peak_source": "measured FFMA microbenchmark on this GPU"}
        del bt
        line["adjoint_roofline"] = {"bound": "hbm", "kernel": "adjoint (runs, sort, per-cell terms, sums)",
                            "achieved": adj_bytes / (sum(bwd) / len(bwd) * 1e-3) / 1e9,
                            "peak": hbm, "unit": "GB/s",
                            "frac": adj_bytes / (sum(bwd) / len(bwd) * 1e-3) / 1e9 / hbm,
                            "traffic": None,
                            "work": f"{adj_bytes:.4g} algorithmic bytes per adjoint (checkpoint 6 B "
                                    "+ dL/dsdf 8 B per cell, points and gradient 48 B per point, "
                                    "triangles 12 B)",
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
        # end to end: host vertices in, host gradient out, through the public torch API
        e2e_t = []
        host_pts = torch.tensor(pts).pin_memory()
        for i in range(1 + min(args.steps, 3)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            vd = host_pts.to("cuda", non_blocking=True)
            s_, o_, t_, r_ = plan.forward(vd)
            gs = 2.0 * w * (s_ - t)
            gr = plan.backward(vd, o_, t_, r_, gs).cpu()
            if i:
                e2e_t.append(time.perf_counter() - t0)
        line["e2e"] = {"value": cells / (sum(e2e_t) / len(e2e_t)), "unit": UNIT,
                       "h2d_bytes_per_step": int(pts.nbytes), "d2h_bytes_per_step": int(gr.numel() * 8),
                       "call": "SDFPlan.forward + SDFPlan.backward (cmg_sdf_plan_*), host vertices in, "
                               "host gradient out"}
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline(pts, tris, (tuple(g.corner), g.spacing, g.dims),
                                                seconds=args.cpu_seconds, probe=48)
            line["cpu_baseline"]["sample"] += " (forward only: the reference has no adjoint)"
        print(json.dumps(line), flush=True)
    barrier(world)


def _measured_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


STREAM_N = 100_000_000
STREAM_CHUNK = 10_000_000


def _stream_soa(kind, n, seed, near=0.0):
    """n queries built in chunks (bounded host memory for the generator): 10 %
    exactly degenerate, `near` within a few ulps of a tie, the rest uniform."""
    from cybermeshgenerator_gb300 import workloads as W
    rows = 12 if kind == "orient3d" else 15
    out = np.empty((rows, n), dtype=np.float64)
    for c0 in range(0, n, STREAM_CHUNK):
        m = min(STREAM_CHUNK, n - c0)
        out[:, c0:c0 + m] = W.predicate_stream(m, kind, degenerate=0.1, near=near,
                                               seed=seed + c0 // STREAM_CHUNK)
    return out


def run_stream(args):
    import torch
    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import build as B
    if rank == 0 or world == 1:
        B.build()
    barrier(world)
    n = args.stream_n
    dev, outs, host = {}, {}, {}
    for kind, seed in (("orient3d", 1000), ("insphere", 2000)):
        host[kind] = _stream_soa(kind, n, seed)
        dev[kind] = torch.from_numpy(host[kind]).to("cuda")
        outs[kind] = torch.empty(n, dtype=torch.int8, device="cuda")
    stream = torch.cuda.current_stream()
    sid = stream.cuda_stream
    stats = {}
    fp32_ms = []  # per step: device time of the two FP32 passes (the library's CUDA events)

    def step(mode=cm.PRED_COMPAT):
        t = 0.0
        for kind, fn in (("orient3d", cm.orient3d_stream), ("insphere", cm.insphere_stream)):
            d = dev[kind]
            _, stats[kind] = fn(([d[k].data_ptr() for k in range(d.shape[0])], n,
                                 outs[kind].data_ptr()), mode, stream=sid)
            t += stats[kind]["fp32_pass_ms"]
        fp32_ms.append(t)

    l0 = cm.gpu_launches()
    barrier(world)
    with Clocks(local) as clk:
        ms = _events_time(torch, stream, step, args.steps, args.warmup)
    barrier(world)
    launches = (cm.gpu_launches() - l0) // (args.steps + args.warmup)
    total_ms = max_over_ranks(sum(ms), world)
    q = 2 * n
    value = q * world * args.steps / (total_ms * 1e-3)
    config = {"workload": f"{n} orient3d + {n} insphere queries, SoA float64 in HBM, 10% exactly "
                          "coplanar/cospherical (small integers scaled by powers of two), the rest "
                          "uniform in [0,1)^3; reference semantics (rounded determinant's sign "
                          "unless exactly zero)",
              "queries": q, "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"}
    line = _base_line(STREAM_METRIC, "queries/s", value, world, args, total_ms, "fp32+fp64+exact",
                      config, launches, clk.summary())
    if rank == 0:
        ex = _events_time(torch, stream, lambda: step(cm.PRED_EXACT), 2, 1)
        line["exact_mode"] = {"value": q * len(ex) / (sum(ex) * 1e-3), "unit": "queries/s",
                              "stats": {k: dict(v) for k, v in stats.items()}}
        step()
        torch.cuda.synchronize()
        line["compat_stats"] = {k: dict(v) for k, v in stats.items()}
        # parity on a sample against the oracle
        import oracle
        orc = oracle.Oracle()
        rng = np.random.default_rng(3)
        ok = True
        for kind in ("orient3d", "insphere"):
            idx = np.sort(rng.choice(n, size=200_000, replace=False))
            want = orc.stream(kind, np.ascontiguousarray(host[kind][:, idx]), oracle.COMPAT)
            ok = ok and bool(np.array_equal(outs[kind].cpu().numpy()[idx], want))
        line["sample_parity"] = {"queries": 400_000, "equal": ok}
        # the harder mix: the same plus 10 % of queries within a few ulps of a tie
        # (the first 2e7 of each kind, replaced in place and restored afterwards)
        m = min(2 * STREAM_CHUNK, n)
        hard_stats, hard_ms = {}, 0.0
        for kind, fn, seed in (("orient3d", cm.orient3d_stream, 3000),
                               ("insphere", cm.insphere_stream, 4000)):
            hs = torch.from_numpy(_stream_soa(kind, m, seed, near=STREAM_NEAR)).to("cuda")
            keep = dev[kind][:, :m].clone()
            dev[kind][:, :m] = hs
            d = dev[kind]
            call = lambda: fn(([d[k].data_ptr() for k in range(d.shape[0])], m,
                               outs[kind].data_ptr()), cm.PRED_COMPAT, stream=sid)
            t = _events_time(torch, stream, call, 2, 1)
            hard_ms += sum(t) / len(t)
            hard_stats[kind] = dict(call()[1])
            dev[kind][:, :m] = keep
        line["near_ties_mix"] = {"value": 2 * m / (hard_ms * 1e-3), "unit": "queries/s",
                                 "queries": 2 * m, "near": STREAM_NEAR, "stats": hard_stats}
        hbm = _measured_hbm()
        byts = n * (96 + 1) + n * (120 + 1)
        t_step = total_ms / args.steps / world * 1e-3
        timed = fp32_ms[args.warmup:args.warmup + args.steps]
        t_fp32 = sum(timed) / len(timed) * 1e-3
        line["roofline"] = {"bound": "hbm", "kernel": "k_pred_fp32_tma<orient3d> + <insphere> "
                                                      "(certification passes, TMA-staged)",
                            "achieved": byts / t_fp32 / 1e9, "peak": hbm, "unit": "GB/s",
                            "frac": byts / t_fp32 / 1e9 / hbm,
                            "traffic": (lambda q: q and n * (q[0] + q[1]))(stream_traffic_per_query()),
                            "traffic_basis": "DRAM bytes of both FP32 launches of a step: the ncu "
                                             "bytes per query of a 2e7-query capture (the "
                                             "traffic grows with the queries) times the queries",
                            "kernel_ms": t_fp32 * 1e3,
                            "step_achieved": byts / t_step / 1e9,
                            "work": "97 B per orient3d + 121 B per insphere query (coordinates read "
                                    "once, sign written once); kernel time from CUDA events the "
                                    "library records around the FP32 passes on the launch stream",
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
        # end to end: host arrays in, host signs out, through the public call
        e2e_t = []
        for i in range(7):
            t0 = time.perf_counter()
            cm.orient3d_stream(host["orient3d"], cm.PRED_COMPAT)
            cm.insphere_stream(host["insphere"], cm.PRED_COMPAT)
            if i >= 2:
                e2e_t.append(time.perf_counter() - t0)
        line["e2e"] = {"value": q / (sum(e2e_t) / len(e2e_t)), "unit": "queries/s",
                       "h2d_bytes_per_step": int(n * (96 + 120)), "d2h_bytes_per_step": int(2 * n),
                       "call": "cmg_orient3d_stream + cmg_insphere_stream, host arrays (read by the "
                               "device through the host's page tables where it can, else copied in "
                               "chunks); signs into pooled page-locked host arrays; mean of 5 steps after 2 "
                               "warm-up steps",
                       "step_s": [round(t, 4) for t in e2e_t],
                       "host_link": os.environ.get("CMG_HOST_STREAM", "pull where supported")}
        if not args.no_cpu:
            line["cpu_baseline"] = _stream_cpu(host, args.cpu_seconds)
        print(json.dumps(line), flush=True)
    barrier(world)


def _stream_cpu(host, seconds, threads=None):
    """The oracle's predicate stream (reference semantics) on all host threads, on
    a contiguous sample of each kind sized to the time budget."""
    import oracle
    orc = oracle.Oracle()
    threads = threads or os.cpu_count() or 1
    tot_q, tot_t = 0, 0.0
    for kind in ("orient3d", "insphere"):
        m = 200_000
        t0 = time.perf_counter()
        orc.stream(kind, np.ascontiguousarray(host[kind][:, :m]), oracle.COMPAT, threads=threads)
        per = (time.perf_counter() - t0) / m
        m = int(min(host[kind].shape[1], max(m, seconds / 2 / per)))
        t0 = time.perf_counter()
        orc.stream(kind, np.ascontiguousarray(host[kind][:, :m]), oracle.COMPAT, threads=threads)
        tot_t += time.perf_counter() - t0
        tot_q += m
    return {"value": tot_q / tot_t, "unit": "queries/s", "cores": int(threads), "kind": "port",
            "sample": f"{tot_q} queries (the first of each kind), reference semantics"}


STL_METRIC = "triangles/s, binary STL read + coincident-vertex merge (2.56M triangles)"


def _stl_workload():
    """The scale workload's 2000 ellipsoids as a binary STL image (2.56M triangles,
    128 MB) and the same surface as ASCII (the first 200 ellipsoids, 256k triangles)."""
    from cybermeshgenerator_gb300 import workloads as W
    pts, tris = W.ellipsoid_field()
    ascii_tris = tris[: 200 * 1280]
    return W.stl_binary(pts, tris), W.stl_ascii(pts, ascii_tris, fmt="{:.9g}"), len(tris), len(ascii_tris)


def _stl_cpu(data, ntris, seconds, reps=1):
    """The oracle's restatement of the reference reader (single thread, as the
    reference's) on the image: triangles/s."""
    import oracle
    orc = oracle.Oracle()
    t0 = time.perf_counter()
    n = 0
    while True:
        orc.stl_read(data)
        n += 1
        if n >= reps or time.perf_counter() - t0 > seconds:
            break
    return ntris * n / (time.perf_counter() - t0)


def run_stl(args):
    import torch
    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import build as B
    if rank == 0 or world == 1:
        B.build()
    barrier(world)
    data, adata, ntris, antris = _stl_workload()
    for _ in range(args.warmup):
        cm.plc_from_stl(data)
    l0 = cm.gpu_launches()
    merge_ms, wall = [], []
    barrier(world)
    with Clocks(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            plc = cm.plc_from_stl(data)
            wall.append(time.perf_counter() - t0)
            merge_ms.append(cm.stl_last_timing()["merge_ms"])
    barrier(world)
    launches = (cm.gpu_launches() - l0) // args.steps
    total_ms = max_over_ranks(sum(merge_ms), world)
    value = ntris * world * args.steps / (total_ms * 1e-3)
    npts = plc.num_points
    config = {"workload": f"binary STL image of the 2000-ellipsoid field ({ntris} triangles, "
                          f"{len(data)} bytes, {npts} merged points): records decoded and "
                          "coincident vertices merged; value from the device phase (records "
                          "resident in HBM), e2e from host image to host PLC arrays",
              "triangles": int(ntris), "bytes": len(data), "points": int(npts),
              "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"}
    line = _base_line(STL_METRIC, "triangles/s", value, world, args, total_ms, "fp32->fp64",
                      config, launches, clk.summary())
    if rank == 0:
        tm = cm.stl_last_timing()
        hbm = _measured_hbm()
        # algorithmic bytes: the 50-byte records read, merged points (24 B) and
        # triangles (12 B) written
        byts = 50 * ntris + 24 * npts + 12 * ntris
        ach = byts / (sum(merge_ms) / len(merge_ms) * 1e-3) / 1e9
        line["roofline"] = {"bound": "hbm", "kernel": "decode + merge (k_stl_extract, k_weld_*)",
                            "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                            "traffic": None, "phase_ms": tm,
                            "work": "50 B per triangle read, 24 B per merged point and 12 B per "
                                    "triangle written",
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
        line["e2e"] = {"value": ntris / (sum(wall) / len(wall)), "unit": "triangles/s",
                       "h2d_bytes_per_step": len(data),
                       "d2h_bytes_per_step": int(24 * npts + 12 * ntris),
                       "call": "cmg_plc_from_stl (host image -> PLC handle)"}
        t0 = time.perf_counter()
        aplc = cm.plc_from_stl(adata)
        ta = time.perf_counter() - t0
        line["ascii"] = {"value": antris / ta, "unit": "triangles/s", "triangles": int(antris),
                         "bytes": len(adata), "phase_ms": cm.stl_last_timing(),
                         "host_threads": os.cpu_count(),
                         "note": "parsed on host threads, merged on the GPU"}
        if not args.no_cpu:
            v = _stl_cpu(data, ntris, args.cpu_seconds)
            line["cpu_baseline"] = {"value": v, "unit": "triangles/s", "cores": 1, "kind": "port",
                                    "sample": "the whole binary image, read by the oracle's "
                                              "restatement of the reference reader (ordered map)"}
            line["ascii"]["cpu_baseline"] = _stl_cpu(adata, antris, args.cpu_seconds)
        del aplc
        print(json.dumps(line), flush=True)
    barrier(world)


def ref_stl(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import oracle
    oracle.build()
    data, _, ntris, _ = _stl_workload()
    v = _stl_cpu(data, ntris, args.cpu_seconds, reps=max(1, args.steps))
    base = {"value": v, "unit": "triangles/s", "cores": 1, "kind": "port",
            "sample": "the whole binary image per step"}
    print(json.dumps(_ref_line(STL_METRIC, "triangles/s", v, args,
                               {"workload": "binary STL of the 2000-ellipsoid field",
                                "parallelism": "1 cpu thread (the reference reader is serial)"},
                               base, ntris)), flush=True)


DETECT_METRIC = "triangles/s, self-intersection preflight (2.56M triangles, all-pairs semantics)"


def _detect_cpu(pts, tris, seconds):
    """The oracle's all-pairs restatement of the reference's self_intersections on the
    first m triangles (m sized to the budget): pair tests/s, extrapolated to the whole
    mesh's T(T-1)/2 pairs (the reference's cost)."""
    import oracle
    orc = oracle.Oracle()
    m = 2000
    t0 = time.perf_counter()
    orc.self_intersections(pts, tris[:m])
    dt = time.perf_counter() - t0
    m = int(min(len(tris), m * max(1.0, (seconds / max(dt, 1e-6)) ** 0.5)))
    t0 = time.perf_counter()
    orc.self_intersections(pts, tris[:m])
    dt = time.perf_counter() - t0
    pair_rate = m * (m - 1) / 2 / dt
    T = len(tris)
    return T / (T * (T - 1) / 2 / pair_rate), m


def run_detect(args):
    import torch
    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import build as B
    if rank == 0 or world == 1:
        B.build()
    barrier(world)
    pts, tris = _scale_workload()
    plc = cm.PLC.from_arrays(pts, tris)
    for _ in range(args.warmup):
        cm.self_intersections(plc)
    l0 = cm.gpu_launches()
    dev_ms, wall = [], []
    barrier(world)
    with Clocks(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            hits = cm.self_intersections(plc)
            wall.append(time.perf_counter() - t0)
            dev_ms.append(float(cm._clib.cmg_self_intersections_last_ms()))
    barrier(world)
    launches = (cm.gpu_launches() - l0) // args.steps
    total_ms = max_over_ranks(sum(dev_ms), world)
    T = len(tris)
    value = T * world * args.steps / (total_ms * 1e-3)
    config = {"workload": f"the 2000-ellipsoid field ({T} triangles, disjoint): every pair of "
                          "triangles sharing no vertex tested for crossing (grid broad phase, "
                          "Guigue-Devillers on the reference's orient3d signs); value from the "
                          "device phase, e2e through cmg_plc_self_intersections",
              "triangles": int(T), "hits": int(len(hits)), "l2": "inputs larger than L2",
              "parallelism": f"replicas x{world}"}
    line = _base_line(DETECT_METRIC, "triangles/s", value, world, args, total_ms, "fp64+exact",
                      config, launches, clk.summary())
    if rank == 0:
        hbm = _measured_hbm()
        byts = T * (12 + 72)  # indices + the three vertices read once per triangle
        ach = byts / (sum(dev_ms) / len(dev_ms) * 1e-3) / 1e9
        line["roofline"] = {"bound": "hbm", "kernel": "k_det_boxes + k_det_bin + k_det_pairs",
                            "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                            "traffic": None, "device_ms": sum(dev_ms) / len(dev_ms),
                            "work": "84 B per triangle (indices and vertices read once); the pair "
                                    "tests are orient3d signs on nearby triangles",
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
        line["e2e"] = {"value": T / (sum(wall) / len(wall)), "unit": "triangles/s",
                       "h2d_bytes_per_step": int(pts.nbytes + tris.astype(np.int32).nbytes),
                       "d2h_bytes_per_step": 8, "call": "cmg_plc_self_intersections (PLC handle)"}
        if not args.no_cpu:
            v, m = _detect_cpu(pts, tris, args.cpu_seconds)
            line["cpu_baseline"] = {"value": v, "unit": "triangles/s", "cores": 1, "kind": "port",
                                    "sample": f"all pairs of the first {m} triangles timed, the pair "
                                              f"rate extrapolated to the {T}-triangle mesh's "
                                              "T(T-1)/2 pairs (extrapolated)"}
        print(json.dumps(line), flush=True)
    barrier(world)


def ref_detect(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import oracle
    oracle.build()
    pts, tris = _scale_workload()
    v, m = _detect_cpu(pts, tris, max(10.0, args.cpu_seconds))
    base = {"value": v, "unit": "triangles/s", "cores": 1, "kind": "port",
            "sample": f"all pairs of the first {m} triangles, extrapolated to T(T-1)/2 pairs"}
    print(json.dumps(_ref_line(DETECT_METRIC, "triangles/s", v, args,
                               {"workload": "self-intersections of the 2000-ellipsoid field",
                                "parallelism": "1 cpu thread (the reference loop is serial)"},
                               base, len(tris))), flush=True)


SIMPLIFY_METRIC = "input triangles/s, grid vertex clustering (2.56M triangles, grid 34)"


def _simplify_cpu(pts, tris, grid, seconds, reps=1):
    """The oracle's restatement of the reference's simplify (single thread, as the
    reference's) on the whole surface: input triangles/s."""
    import oracle
    orc = oracle.Oracle()
    t0 = time.perf_counter()
    n = 0
    while True:
        orc.simplify(pts, tris, grid)
        n += 1
        if n >= reps or time.perf_counter() - t0 > seconds:
            break
    return len(tris) * n / (time.perf_counter() - t0)


def run_simplify(args):
    import torch
    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import build as B
    if rank == 0 or world == 1:
        B.build()
    barrier(world)
    pts, tris = _scale_workload()
    plc = cm.PLC.from_arrays(pts, tris)
    grid = 34
    for _ in range(args.warmup):
        cm.simplify(plc, grid)
    l0 = cm.gpu_launches()
    dev_ms, wall = [], []
    barrier(world)
    with Clocks(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            out = cm.simplify(plc, grid)
            wall.append(time.perf_counter() - t0)
            dev_ms.append(cm.simplify_last_timing()["cluster_ms"])
    barrier(world)
    launches = (cm.gpu_launches() - l0) // args.steps
    total_ms = max_over_ranks(sum(dev_ms), world)
    T, P = len(tris), len(pts)
    value = T * world * args.steps / (total_ms * 1e-3)
    nrep, nkept = out.num_points, len(out.triangles)
    config = {"workload": f"the 2000-ellipsoid field ({T} triangles, {P} points) simplified at "
                          f"the reference's default grid {grid} ({nrep} representatives, {nkept} "
                          "triangles kept); value from the device phase (points and facets "
                          "resident in HBM), e2e through cmg_plc_simplify (host PLC to host PLC)",
              "triangles": int(T), "points": int(P), "grid": grid, "representatives": int(nrep),
              "kept": int(nkept), "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"}
    line = _base_line(SIMPLIFY_METRIC, "triangles/s", value, world, args, total_ms, "fp64",
                      config, launches, clk.summary())
    if rank == 0:
        hbm = _measured_hbm()
        # algorithmic bytes: points (24 B) and facets (12 B indices + 8 B offset) read
        # once, representatives (24 B) and kept triangles (12 B) written
        byts = 24 * P + 20 * T + 24 * nrep + 12 * nkept
        ach = byts / (sum(dev_ms) / len(dev_ms) * 1e-3) / 1e9
        line["roofline"] = {"bound": "hbm", "kernel": "clustering (k_bbox .. k_tri_out, 13 kernels "
                                                      "+ scans and the radix sort)",
                            "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                            "traffic": None, "phase_ms": cm.simplify_last_timing(),
                            "work": "24 B per point and 20 B per facet read, 24 B per "
                                    "representative and 12 B per kept triangle written",
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
        line["e2e"] = {"value": T / (sum(wall) / len(wall)), "unit": "triangles/s",
                       "h2d_bytes_per_step": int(24 * P + 20 * T + 8),
                       "d2h_bytes_per_step": int(24 * nrep + 12 * nkept),
                       "call": "cmg_plc_simplify (PLC handle -> PLC handle)"}
        # a fine grid keeps most triangles: the dedupe table and output dominate
        # (1 warm-up call, then the mean of 3)
        fine = cm.simplify(plc, 512)
        tf, cl = [], []
        for _ in range(3):
            del fine
            t0 = time.perf_counter()
            fine = cm.simplify(plc, 512)
            tf.append(time.perf_counter() - t0)
            cl.append(cm.simplify_last_timing()["cluster_ms"])
        line["grid512"] = {"device_triangles_per_s": T / (sum(cl) / len(cl) * 1e-3),
                           "e2e_triangles_per_s": T / (sum(tf) / len(tf)),
                           "representatives": int(fine.num_points),
                           "kept": int(len(fine.triangles))}
        if not args.no_cpu:
            v = _simplify_cpu(pts, tris, grid, args.cpu_seconds)
            line["cpu_baseline"] = {"value": v, "unit": "triangles/s", "cores": 1, "kind": "port",
                                    "sample": "the whole surface at grid 34, simplified by the "
                                              "oracle's restatement of the reference's simplify"}
            line["grid512"]["cpu_baseline"] = _simplify_cpu(pts, tris, 512, args.cpu_seconds)
        print(json.dumps(line), flush=True)
    barrier(world)


def ref_simplify(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import oracle
    oracle.build()
    pts, tris = _scale_workload()
    v = _simplify_cpu(pts, tris, 34, args.cpu_seconds, reps=max(1, args.steps))
    base = {"value": v, "unit": "triangles/s", "cores": 1, "kind": "port",
            "sample": "the whole surface at grid 34 per step"}
    print(json.dumps(_ref_line(SIMPLIFY_METRIC, "triangles/s", v, args,
                               {"workload": "simplify of the 2000-ellipsoid field at grid 34",
                                "parallelism": "1 cpu thread (the reference is serial)"},
                               base, len(tris))), flush=True)


SIZING_METRIC = "queries/s, background sizing field (663,552-tetrahedron field, 1e7 queries)"
SIZING_TEST_FLOPS = 96  # one containment test: four orient3d determinants (23 flops) + four divides


def _sizing_workload(n=10_000_000):
    """A 48^3-cell Kuhn background mesh of the unit cube (663,552 tetrahedra, 117,649
    nodes, interior nodes jittered by 0.3 cells) with random node sizes, and n queries:
    half uniform over the box grown by 10 % per side (about 42 % of those outside the
    mesh), the rest on nodes, edge midpoints and face centroids."""
    from cybermeshgenerator_gb300 import workloads as W
    P, T = W.kuhn_tet_mesh(48, 0.3, seed=11)
    S = np.random.default_rng(11).uniform(0.01, 0.2, len(P))
    Q = W.sizing_queries(P, T, n, seed=12)
    return P, T, S, Q


def _sizing_cpu(P, T, S, Q, seconds, threads=None):
    """The oracle's restatement of the reference's closure (a scan of every tetrahedron
    per query) on all host threads, over a random sample of the queries sized to the
    budget: queries/s."""
    import oracle
    orc = oracle.Oracle()
    rng = np.random.default_rng(5)
    m = 64
    while True:
        idx = rng.choice(len(Q), m, replace=False)
        t0 = time.perf_counter()
        orc.sizing(P, T, S, 1.0, Q[idx], threads=threads)
        dt = time.perf_counter() - t0
        if dt > seconds / 4 or m >= len(Q):
            return m / dt, m, orc.threads(threads)
        m = int(min(len(Q), m * max(2.0, seconds / max(dt, 1e-3) / 2)))


def run_sizing(args):
    import torch
    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import cybermeshgenerator_gb300 as cm
    from cybermeshgenerator_gb300 import build as B
    if rank == 0 or world == 1:
        B.build()
    barrier(world)
    P, T, S, Q = _sizing_workload()
    n = len(Q)
    t0 = time.perf_counter()
    field = cm.SizingField(P, T, S, 1.0)
    build_s = time.perf_counter() - t0
    dq = torch.from_numpy(Q).cuda()
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        field.eval(dq)
    torch.cuda.synchronize()
    l0 = cm.gpu_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier(world)
    with Clocks(local) as clk:
        for a, b in ev:
            a.record(stream)
            out = field.eval(dq)
            b.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    launches = (cm.gpu_launches() - l0) // args.steps
    dev_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = max_over_ranks(sum(dev_ms), world)
    value = n * world * args.steps / (total_ms * 1e-3)
    st = field.stats()
    config = {"workload": f"background sizing field of a 48^3-cell Kuhn mesh ({len(T)} "
                          f"tetrahedra, {len(P)} nodes) at {n} queries (half uniform over the "
                          "box grown by 10 %, half on nodes, edge midpoints and face centroids); "
                          "value from the device evaluation (queries resident in HBM), e2e "
                          "through cmg_sizing_eval with host arrays",
              "tetrahedra": int(len(T)), "nodes": int(len(P)), "queries": int(n),
              "inside": int(st["inside"]), "nearest": int(st["nearest"]), "slow": int(st["slow"]),
              "global_tets": int(st["global_tets"]), "far_tets": int(st["far_tets"]),
              "cell_entries": int(st["binned_pairs"]),
              "build_s": build_s, "l2": "inputs larger than L2",
              "parallelism": f"replicas x{world}"}
    line = _base_line(SIZING_METRIC, "queries/s", value, world, args, total_ms, "fp64",
                      config, launches, clk.summary())
    if rank == 0:
        p64 = cm.peak_flops(True)
        flops = st["tests"] * SIZING_TEST_FLOPS
        ms = sum(dev_ms) / len(dev_ms)
        ach, frac = fraction_of_peak(flops, ms, p64)
        line["roofline"] = {"bound": "fp64", "kernel": "k_sizing_eval (+ k_sizing_slow)",
                            "achieved": ach / 1e12, "peak": p64 / 1e12, "unit": "TFLOP/s",
                            "frac": frac, "traffic": None,
                            "tests_per_query": st["tests"] / n,
                            "candidates_per_query": st["candidates"] / n,
                            "work": f"{SIZING_TEST_FLOPS} flops per full containment test "
                                    "(four orient3d determinants + four divides), tests counted "
                                    "on the device",
                            "peak_source": "measured DFMA microbenchmark (FMA = 2 flops)"}
        wall = []
        for i in range(2 + max(1, min(args.steps, 3))):  # 2 warm-up calls
            t0 = time.perf_counter()
            host = field.eval(Q)
            if i >= 2:
                wall.append(time.perf_counter() - t0)
        assert np.array_equal(host.view(np.uint64), out.cpu().numpy().view(np.uint64))
        line["e2e"] = {"value": n / (sum(wall) / len(wall)), "unit": "queries/s",
                       "h2d_bytes_per_step": int(Q.nbytes), "d2h_bytes_per_step": int(8 * n),
                       "call": "cmg_sizing_eval (host queries -> host sizes, pooled page-locked "
                               "result); mean of 3 calls after 2 warm-up calls",
                       "phase_ms": {k: field.stats()[k] for k in ("upload_ms", "eval_ms", "download_ms")}}
        if not args.no_cpu:
            v, m, th = _sizing_cpu(P, T, S, Q, args.cpu_seconds)
            line["cpu_baseline"] = {"value": v, "unit": "queries/s", "cores": th, "kind": "port",
                                    "sample": f"{m} random queries of the workload, each scanning "
                                              "the tetrahedra in order as the reference's closure"}
        print(json.dumps(line), flush=True)
    barrier(world)


def ref_sizing(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import oracle
    oracle.build()
    P, T, S, Q = _sizing_workload()
    v, m, th = _sizing_cpu(P, T, S, Q, max(10.0, args.cpu_seconds))
    base = {"value": v, "unit": "queries/s", "cores": th, "kind": "port",
            "sample": f"{m} random queries of the workload"}
    print(json.dumps(_ref_line(SIZING_METRIC, "queries/s", v, args,
                               {"workload": "background sizing field, 663,552 tetrahedra",
                                "parallelism": "cpu threads"}, base, len(Q))), flush=True)


def _ref_line(metric, unit, value, args, config, base, units_per_step):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return {"impl": "reference", "metric": metric, "value": value, "unit": unit, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": units_per_step / value * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic", "config": config, "cpu_baseline": base,
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def ref_batch(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import oracle
    oracle.build()
    items = _batch_workload()
    base = _batch_cpu(items, max(10.0, min(60.0, args.cpu_seconds * 2)))
    orc = oracle.Oracle()
    cells = sum(orc.make_grid(b.points, b.resolution, b.pad).ncell for b in items)
    print(json.dumps(_ref_line(BATCH_METRIC, UNIT, base["value"], args,
                               {"workload": "batch of 512 meshes (see the ours line)",
                                "parallelism": "cpu threads"}, base, cells)), flush=True)


def ref_scale(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import oracle
    oracle.build()
    pts, tris = _scale_workload()
    g = oracle.Oracle().make_grid(pts, 510, 1)
    base = cpu_baseline(pts, tris, (tuple(g.corner), g.spacing, g.dims),
                        seconds=max(20.0, args.cpu_seconds), probe=48)
    print(json.dumps(_ref_line(SCALE_METRIC, UNIT, base["value"], args,
                               {"workload": "2000 ellipsoids at 512^3 (forward only: the reference "
                                            "has no adjoint)", "parallelism": "cpu threads"},
                               base, g.ncell)), flush=True)


def ref_stream(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import oracle
    oracle.build()
    host = {k: _stream_soa(k, 4 * STREAM_CHUNK // 10, s) for k, s in (("orient3d", 1000),
                                                                       ("insphere", 2000))}
    base = _stream_cpu(host, args.cpu_seconds)
    print(json.dumps(_ref_line(STREAM_METRIC, "queries/s", base["value"], args,
                               {"workload": "the stream workload's first 4e6 queries of each kind",
                                "parallelism": "cpu threads"}, base, 2 * STREAM_N)), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--brick", type=int, default=0)
    ap.add_argument("--stage", type=int, default=-1,
                    help="mixed record access: 0 L1/L2, 1 staged in shared memory, -1 default")
    ap.add_argument("--walk-warps", type=int, default=0,
                    help="warps per brick of the candidate walk (1, 2, 4); 0 = autotuned")
    ap.add_argument("--probe", type=int, default=0, help="mixed probe head; 0 = autotuned")
    ap.add_argument("--ctas", type=int, default=0,
                    help="evaluation CTAs per SM (12, 16); 0 = autotuned")
    ap.add_argument("--no-autotune", action="store_true",
                    help="library defaults for every tunable not given")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--stream-n", type=int, default=STREAM_N,
                    help="queries per kind of the stream workload (smaller for profiler captures)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="sdf",
                    choices=["sdf", "batch", "scale", "stream", "stl", "detect", "simplify",
                             "sizing"])
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        {"sdf": run_reference, "batch": ref_batch, "scale": ref_scale,
         "stream": ref_stream, "stl": ref_stl, "detect": ref_detect,
         "simplify": ref_simplify, "sizing": ref_sizing}[args.workload](args)
    else:
        {"sdf": run_ours, "batch": run_batch, "scale": run_scale,
         "stream": run_stream, "stl": run_stl, "detect": run_detect,
         "simplify": run_simplify, "sizing": run_sizing}[args.workload](args)


if __name__ == "__main__":
    main()
