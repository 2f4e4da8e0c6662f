"""Benchmark of the fused geometry evaluation on one GB300 (the driver's contract).

Workload: curved P2 tetrahedra, 64^3 subcells x 6 = 1,572,864 cells (10 nodes each,
2,146,689 nodes), node coordinates mapped by x' = x + 0.05 sin(2 pi y) sin(2 pi z) (cyclic)
plus seeded uniform +-0.02 h jitter of the interior nodes, 24 points per cell; outputs x, J,
det J and K = J^-1 at every point (22 values). One step = one evaluation of the whole block
(one fused launch). `value` is quadrature points per second with the mesh resident on the
device; `e2e` adds, every step, the host-to-device copy of the node and dofmap arrays from
pinned host memory, the evaluation, the measure (sum of det J * w) and its read back.

Modes (`--mode`): `split` (default): the f64 mesh evaluated in FP32 on cell-shifted
coordinates into f32 fields, FP64 recompute at near-degenerate points; its error against the
plain FP64 GPU path is measured per output in the same run and reported with it, together with
that path's own rate. `f64`: the plain per-block FP64 path. `f32`: an f32 mesh in FP32.

`--impl reference` times the CPU restatement of the reference's f64 evaluation (the oracle,
C + OpenMP) on the host cores over the same workload.

Runs under torchrun for N > 1: every rank evaluates its own copy of the workload (replicas,
weak scaling; the path has no exchange), rank 0 reports the whole-job rate over the slowest
rank's time.
"""

from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent

WORKLOAD = "curved P2 tetrahedra 64^3x6, 24-point rule, fused x/J/detJ/K"
# 24 points: the collapsed Gauss-Jacobi product with 4 x 3 x 2 points (the reference's rules
# have m^3 points; its nearest, gauss_rule(Tet, 4), has 27).
RULE_COUNTS = (4, 3, 2)
METRIC = "Jacobian qpoints/s (fwd, fwd+adjoint) vs plain FP64 GPU path at stated error"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--mode", choices=["split", "f64", "f32"], default="split")
    p.add_argument("--n", type=int, default=64, help="subcells per direction")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def build_mesh(n: int):
    from gridcl_gb300 import meshes

    return meshes.curved_box("Tetrahedron", n, 2, jitter=0.02, seed=2026)


def rule():
    from gridcl_gb300 import refcell

    return refcell.collapsed_rule("Tetrahedron", RULE_COUNTS)


def algorithmic_bytes(cells: int, k: int, nodes: int, gd: int, qpts: int, es: int, nout: int) -> int:
    """Compulsory traffic of one evaluation: the dofmap (4 K bytes per cell), every node once
    (GD values) and every output value once (written)."""
    return cells * k * 4 + nodes * gd * es + qpts * nout * es


class ClockSampler:
    """nvidia-smi samples (SM clock, max clock, throttle reasons) while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None
        self.window = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        time.sleep(1.0)

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), line.strip()))

    def mark(self, t0, t1):
        self.window = (t0, t1)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        rows = []
        for t, line in self.samples:
            if self.window and not (self.window[0] - 0.15 <= t <= self.window[1] + 0.15):
                continue
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[3:]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples in the timed window"]}
        names = ["active_mask", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(1, 5) if r[2][i].lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(mesh, pts, target_s: float = 10.0):
    """The oracle (C + OpenMP, all host threads) over the whole workload, repeated for about
    `target_s` seconds; returns (qpoints/s, threads, passes)."""
    from oracle import oracle as orc

    orc.build()
    cells = mesh.blocks[0].cells
    origin = 0.5 * (mesh.nodes.min(0) + mesh.nodes.max(0))
    absx = (mesh.nodes - origin) + origin  # the stored nodes widened (f64 storage)
    from oracle import refcell as orc_refcell

    tab = orc_refcell.tabulate("Tetrahedron", 2, pts, 1)
    threads = orc.max_threads()
    passes, t0 = 0, time.perf_counter()
    while True:
        orc.eval_block("Tetrahedron", 2, absx, cells, pts, factors=("x", "j", "detj", "k"), tab=tab)
        passes += 1
        el = time.perf_counter() - t0
        if el >= target_s or passes >= 200:
            break
    qpts = cells.shape[0] * pts.shape[0] * passes
    return qpts / el, threads, passes


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mesh = build_mesh(args.n)
    pts, _ = rule()
    from oracle import oracle as orc
    from oracle import refcell as orc_refcell

    orc.build()
    cells = mesh.blocks[0].cells
    tab = orc_refcell.tabulate("Tetrahedron", 2, pts, 1)
    qpts = cells.shape[0] * pts.shape[0]
    for _ in range(args.warmup):
        orc.eval_block("Tetrahedron", 2, mesh.nodes, cells, pts, factors=("x", "j", "detj", "k"), tab=tab)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.eval_block("Tetrahedron", 2, mesh.nodes, cells, pts, factors=("x", "j", "detj", "k"), tab=tab)
    el = time.perf_counter() - t0
    value = qpts * args.steps / el
    threads = orc.max_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "qpoints/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": int(cells.shape[0]), "points": int(pts.shape[0]),
                   "qpoints": int(qpts)},
        "cpu_baseline": {"value": value, "unit": "qpoints/s", "cores": threads, "kind": "port",
                         "sample": f"the whole workload per step ({qpts} qpoints), f64"},
        "e2e": {"value": value, "unit": "qpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_steps(step, steps, flush, stream):
    """CUDA-event time of each step (L2 flushed before each, outside the events); mean ms."""
    import torch

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for i in range(steps):
        flush.zero_()
        starts[i].record(stream)
        step()
        ends[i].record(stream)
    torch.cuda.synchronize()
    times = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    return sum(times) / len(times)


def run_ours(args):
    import torch
    import torch.distributed as dist

    import gridcl_gb300 as tg

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    mesh_dtype = torch.float32 if args.mode == "f32" else torch.float64
    precision = "split" if args.mode == "split" else "native"
    out_es = 8 if args.mode == "f64" else 4

    mesh = build_mesh(args.n)
    pts, w = rule()
    g = tg.Geometry.from_host(mesh, dtype=mesh_dtype)
    ps = tg.PointSet("Tetrahedron", pts, w)
    cells, k = mesh.blocks[0].cells.shape
    nq = pts.shape[0]
    qpts = cells * nq
    factors = ("points", "jacobian", "detj", "pinv")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    out = tg.geometric_factors_block(g, 0, ps, factors, precision=precision, recomputed=count)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        tg.geometric_factors_block(g, 0, ps, factors, out=out, precision=precision, recomputed=count)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall0 = time.time()
    ms = time_steps(step, args.steps, flush, stream)
    t_wall1 = time.time()
    if world > 1:
        dist.barrier()
    sampler.mark(t_wall0, t_wall1)
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())

    # The plain FP64 GPU path on the same mesh: its rate, and the split path's error against it.
    plain = None
    if args.mode == "split":
        ref = tg.geometric_factors_block(g, 0, ps, factors)

        def plain_step():
            tg.geometric_factors_block(g, 0, ps, factors, out=ref)

        plain_step()
        torch.cuda.synchronize()
        plain_ms = time_steps(plain_step, max(3, min(args.steps, 5)), flush, stream)
        errs = {}
        for f in factors:
            a = out[f].chunks[0].data.double()
            b = ref[f].chunks[0].data
            errs[f] = float((a - b).abs().max() / b.abs().max())
        plain = {"ms_per_step": plain_ms, "value": world * qpts / (plain_ms * 1e-3),
                 "rel_err_vs_fp64": errs,
                 "speedup": plain_ms / ms}
        del ref
    recomputed = int(count.item())

    # End to end through the public API: pinned host inputs copied in every step, measure read back.
    host_nodes = g.nodes.cpu().pin_memory()
    host_dofmap = g.blocks[0].dofmap.cpu().pin_memory()
    h2d = host_nodes.numel() * host_nodes.element_size() + host_dofmap.numel() * 4
    e2e_steps = max(3, min(args.steps, 10))
    meas_geom = g

    def e2e_step():
        g.nodes.copy_(host_nodes, non_blocking=True)
        g.blocks[0].dofmap.copy_(host_dofmap, non_blocking=True)
        f = tg.geometric_factors_block(g, 0, ps, factors, out=out, precision=precision)
        return measure_of(tg, meas_geom, ps, f["detj"])

    for _ in range(2):
        vol = e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        vol = e2e_step()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) / e2e_steps * 1e3
    t = torch.tensor([e2e_ms], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_ms = float(t.item())
    sampler.stop()

    if rank == 0:
        nout = 3 + 9 + 1 + 9
        node_es = 4 if args.mode == "f32" else 8
        alg = cells * k * 4 + g.nodes.shape[0] * 3 * node_es + qpts * nout * out_es
        peaks = {}
        try:
            peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        except (OSError, ValueError):
            pass
        peak = float(peaks.get("hbm_gbs", 6800.0))
        achieved = alg / (ms * 1e-3) / 1e9
        dtype = {"split": "f32", "f64": "f64", "f32": "f32"}[args.mode]
        line = {
            "metric": METRIC, "value": world * qpts / (ms_max * 1e-3), "unit": "qpoints/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic (seeded sin-mapped, jittered P2 tetrahedral box)",
            "config": {"workload": WORKLOAD, "mode": args.mode, "mesh_dtype": str(mesh_dtype),
                       "cells": int(cells), "nodes_per_cell": int(k),
                       "nodes": int(g.nodes.shape[0]), "points": int(nq), "qpoints": int(qpts),
                       "outputs_per_qpoint": nout, "output_bytes": out_es, "tile": 16,
                       "l2": "256 MiB flush between steps (outside the timed events); outputs exceed L2",
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None,
                         "algorithmic_bytes_per_launch": alg,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if "hbm_gbs" in peaks else "fallback 6800"},
            "e2e": {"value": world * qpts / (e2e_ms * 1e-3), "unit": "qpoints/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": out_es, "ms_per_step": e2e_ms,
                    "measure": vol},
            "gpu_launches": args.steps,
            "clocks": sampler.summary(),
        }
        if plain is not None:
            line["plain_fp64_gpu"] = plain
            line["recomputed_points"] = recomputed
        if not args.no_cpu_baseline:
            v, threads, passes = cpu_baseline(mesh, pts)
            line["cpu_baseline"] = {"value": v, "unit": "qpoints/s", "cores": threads, "kind": "port",
                                    "sample": f"{passes} passes over the whole workload (f64), about 10 s"}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def measure_of(tg, g, ps, detj):
    """The measure from a det J field (f32 or f64) through the native sum tree."""
    import torch

    from gridcl_gb300._lib import check, lib
    from gridcl_gb300.geometry import current_stream_handle

    dt = detj.chunks[0].data.dtype
    es = 4 if dt == torch.float32 else 8
    sums = torch.empty(detj.num_cells, dtype=dt, device="cuda")
    wd = ps.weights_device(dt)
    stream = current_stream_handle()
    ch = detj.chunks[0]
    check(lib().tlg_measure_cell_sums(ch.data.data_ptr(), es, ch.num_cells, detj.num_points, detj.tile,
                                      wd.data_ptr(), sums.data_ptr(), stream))
    nbytes = int(lib().tlg_sum_workspace_bytes(es, detj.num_cells))
    work = torch.empty(max(nbytes, es), dtype=torch.uint8, device="cuda")
    res = torch.empty(1, dtype=dt, device="cuda")
    check(lib().tlg_sum(sums.data_ptr(), es, detj.num_cells, work.data_ptr(), nbytes, res.data_ptr(), stream))
    return float(res.item())


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
