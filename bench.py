"""Benchmark of the fused geometry evaluation on one GB300.

Workload: curved P2 tetrahedra, 64^3 subcells x 6 = 1,572,864 cells (10 nodes each,
2,146,689 nodes), node coordinates mapped by x' = x + 0.05 sin(2 pi y) sin(2 pi z) (cyclic)
plus seeded uniform +-0.02 h jitter of the interior nodes, 24 points per cell; outputs x, J,
det J and K = J^-1 at every point (22 values). One step = one evaluation of the whole block
(one fused launch). `value` is quadrature points per second with the mesh resident on the
device; `e2e` adds, every step, the host-to-device copy of the node and dofmap arrays from
pinned host memory, the evaluation, the measure (sum of det J * w) and its read back.

Modes (`--mode`): `df64` (default): the f64 mesh evaluated into f64 fields in double-float
arithmetic on the FP32 pipe (f64-accurate: errors against the oracle of a few 1e-13, printed as
`error_vs_oracle` over a seeded sample of 65,536 cells). `split`: FP32 arithmetic on cell-shifted
coordinates into f32 fields (errors of about 1e-6), FP64 recompute at near-degenerate points.
`f64`: the plain per-block FP64 path. `f32`: an f32 mesh in FP32. The run also times the other
precisions of an f64 mesh on the same mesh (`plain_fp64_gpu`, `df64_gpu`, `split_gpu`, each with
its errors against the oracle); `vs_baseline` is the line's speed-up over the plain FP64 GPU path
of the same run, the metric's baseline.

`--impl reference` times the CPU restatement of the reference's f64 evaluation (the oracle,
C + OpenMP) on the host cores over the same workload, with the mesh and rule built from the
oracle's reference cells (this arm loads none of the library).

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
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the evaluation
# kernel on the 64^3 workload, measured on a GB300 by one-pass ncu captures of
# `bench.py --no-extras --no-cpu-baseline --steps 3 --warmup 3 [--mode f64]` (-s 3 -c 1):
# split eval_pair_kernel<1,3,3,10> 191.07 MB + 3.26 GB; f64 eval_direct_kernel<double,3,3,10,16>
# 166.22 MB + 6.58 GB; double-float eval_df_kernel<3,3,10> 171.69 MB + 6.581 GB. Reported as
# roofline.traffic, scaled by quadrature points for other n.
NCU_TRAFFIC_64 = {"split": 191.07e6 + 3.26e9, "f64": 166.22e6 + 6.58e9, "df64": 171.69e6 + 6.581e9}
QPOINTS_64 = 64 ** 3 * 6 * 24


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--mode", choices=["df64", "split", "f64", "f32"], default="df64")
    p.add_argument("--n", type=int, default=64, help="subcells per direction")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the other workloads (hybrid batch, hybrid forward + adjoint, sphere surface, "
                        "Q2 adjoint, pull-back, ordering, P1 box)")
    p.add_argument("--workload", choices=["main", *EXTRAS], default="main",
                   help="run one of the other workloads alone and print its JSON object")
    p.add_argument("--adjoint-n", type=int, default=128, help="Q2 hexahedra per direction (adjoint)")
    p.add_argument("--fd-nodes", type=int, default=1000, help="nodes of the adjoint's central-difference check")
    p.add_argument("--hex-n", type=int, default=64, help="hexahedra per direction (hex_strategies)")
    p.add_argument("--ho-n", type=int, default=16, help="subcells per direction (high_order)")
    p.add_argument("--ho-degree", type=int, default=6, help="degree (high_order_case)")
    p.add_argument("--ho-precision", default="f32", choices=("f32", "split", "f64"), help="(high_order_case)")
    return p.parse_args()


def build_mesh(n: int, lagrange_points=None):
    from gridcl_gb300 import meshes

    return meshes.curved_box("Tetrahedron", n, 2, jitter=0.02, seed=2026, lagrange_points=lagrange_points)


def rule():
    from gridcl_gb300 import refcell

    return refcell.collapsed_rule("Tetrahedron", RULE_COUNTS)


SAMPLE_CELLS = 65536  # cells of the seeded sample compared with the oracle at full size


def sample_cells(num_cells: int, count: int = SAMPLE_CELLS, seed: int = 2026) -> np.ndarray:
    """A seeded sample of distinct cell indices (all cells when there are fewer), ascending."""
    if num_cells <= count:
        return np.arange(num_cells)
    return np.sort(np.random.default_rng(seed).choice(num_cells, count, replace=False))


def field_at(field, cells: np.ndarray) -> np.ndarray:
    """Values of a one-chunk QuadField at the given cells, ``[cell][point][component]`` on the host
    (gathered on the device from the tiled layout, field.rs:121-162)."""
    import torch

    t, q, length = field.tile, field.num_points, field.length
    data = field.chunks[0].data
    c = torch.from_numpy(np.asarray(cells, dtype=np.int64)).to(data.device)
    qq = torch.arange(q, device=data.device)
    kk = torch.arange(length, device=data.device)
    idx = (((c // t)[:, None, None] * q + qq[None, :, None]) * length + kk[None, None, :]) * t + (c % t)[:, None, None]
    return data[idx].double().cpu().numpy()


def oracle_sample(mesh, geom, cell: str, degree: int, pts, cells: np.ndarray, block: int = 0,
                  factors=("x", "j", "detj", "k")):
    """The oracle's factors at the given cells (the stored node coordinates plus origin)."""
    from oracle import oracle as orc

    absx = geom.nodes.double().cpu().numpy() + np.array(geom.origin[: geom.gdim])
    return orc.eval_block(cell, degree, absx, mesh.blocks[block].cells[cells], pts, factors=factors)


def errors_vs_oracle(fields: dict, want: dict, cells: np.ndarray) -> dict:
    """max |got - oracle| / max |oracle| per output over the sampled cells."""
    names = {"points": "x", "jacobian": "j", "detj": "detj", "pinv": "k", "normals": "normals"}
    out = {}
    for f, fld in fields.items():
        w = want[names[f]].reshape(len(cells), fld.num_points, -1)
        out[f] = float(np.abs(field_at(fld, cells) - w).max() / np.abs(w).max())
    return out


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
    """The oracle (C + OpenMP restatement of the reference's f64 evaluation) over the workload on
    the host cores. The mesh and the rule come from the oracle's own reference cells, so that this
    arm loads none of the library."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as orc
    from oracle import refcell as orc_refcell

    mesh = build_mesh(args.n, lagrange_points=orc_refcell.lagrange_points)
    pts, _ = orc_refcell.collapsed_rule("Tetrahedron", RULE_COUNTS)

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


def gpu_hold(ms: float = 1.0):
    """Keeps the stream busy for about `ms` (a device spin) so that the host enqueues what follows
    before the GPU reaches it: events recorded next then bracket device work only, not the host's
    launch overhead."""
    import torch

    torch.cuda._sleep(int(ms * 2.0e6))


def max_over_ranks(x: float, device: str = "cuda") -> float:
    """The largest value of `x` over the ranks of the process group (`x` itself without one): the
    slowest rank's time, which the whole-job rate divides by."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: int, world: int, ms: float) -> float:
    """Units per second of the whole job: every rank processes `units_per_rank` (replicas, weak
    scaling) in at most `ms` milliseconds."""
    return world * units_per_rank / (ms * 1e-3)


def time_steps(step, steps, flush, stream):
    """CUDA-event time of each step (L2 flushed before each, outside the events); mean ms."""
    import torch

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for i in range(steps):
        flush.zero_()
        gpu_hold()
        starts[i].record(stream)
        step()
        ends[i].record(stream)
    torch.cuda.synchronize()
    times = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    return sum(times) / len(times)



# ------------------------------------------------------------------------------------------
# The other workloads, measured in the same run and reported under "workloads".

def event_ms(fn, reps: int = 5, warm: int = 2) -> float:
    import torch

    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    gpu_hold(2.0)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def median_launch_ms(fn, n: int = 15) -> float:
    """The median of `n` launches timed one by one with CUDA events (after two untimed ones)."""
    import torch

    fn()
    fn()
    times = []
    for _ in range(n):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
    return float(np.median(times))


def rel_err_fields(a: dict, b: dict) -> dict:
    out = {}
    for k in a:
        x = a[k].chunks[0].data.double()
        y = b[k].chunks[0].data.double()
        out[k] = float((x - y).abs().max() / y.abs().max())
    return out


def extra_hybrid():
    """Hybrid mesh, one graph launch: 2,000,000 Q2 hexahedra (27-point Gauss), 300,000 P2 prisms
    (21 points), 50,000 P3 tetrahedra (24 points); plain per-block FP64 launches against the
    batched FP64, double-float (f64-accurate) and split-precision graphs, each with its errors
    against the oracle on 16,384 seeded cells per block."""
    import torch

    import gridcl_gb300 as tg
    from gridcl_gb300 import meshes, refcell

    mesh = meshes.hybrid_box(2_000_000, 300_000, 50_000)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    sets = [tg.PointSet("Hexahedron", *refcell.gauss_rule("Hexahedron", 4)),
            tg.PointSet("Prism", *refcell.collapsed_rule("Prism", (3, 1, 7))),
            tg.PointSet("Tetrahedron", *refcell.collapsed_rule("Tetrahedron", (4, 3, 2)))]
    rule = tg.QuadRule(sets)
    qpts = sum(b.num_cells * len(rule.get(b.element.cell)) for b in g.blocks)
    factors = ("points", "jacobian", "detj", "pinv")
    plain_out = [tg.geometric_factors_block(g, b, rule.get(blk.element.cell), factors)
                 for b, blk in enumerate(g.blocks)]

    def plain():
        for b, blk in enumerate(g.blocks):
            tg.geometric_factors_block(g, b, rule.get(blk.element.cell), factors, out=plain_out[b])

    plain_ms = event_ms(plain, reps=3, warm=1)
    res = {"workload": "hybrid: 2,000,000 Q2 hex (27 pts) + 300,000 P2 prisms (21) + 50,000 P3 tets (24), "
                       "sin-mapped + jittered, fused x/J/detJ/K", "qpoints": int(qpts),
           "plain_fp64_per_block": {"ms": plain_ms, "value": qpts / (plain_ms * 1e-3)}}
    samples = [sample_cells(b.num_cells, 16384, seed=7 + i) for i, b in enumerate(g.blocks)]
    want = [oracle_sample(mesh, g, blk.element.cell, blk.element.degree, rule.get(blk.element.cell).points, samples[b],
                          block=b) for b, blk in enumerate(g.blocks)]
    res["plain_fp64_per_block"]["error_vs_oracle"] = {
        b: errors_vs_oracle(plain_out[b], want[b], samples[b]) for b in range(len(g.blocks))}
    for precision in ("native", "df64", "split"):
        batch = tg.Batch(g, rule, factors=factors, precision=precision)
        batch.tune()
        ms = event_ms(batch.launch, reps=10)
        single = median_launch_ms(batch.launch, 15)
        key = {"native": "batched_fp64_graph", "df64": "batched_df64_graph", "split": "batched_split_graph"}[precision]
        res[key] = {"ms": ms, "value": qpts / (ms * 1e-3), "tuning": batch.tuning(),
                    "median_single_launch_ms": single,
                    "speedup_vs_plain_fp64": plain_ms / ms,
                    "error_vs_oracle": {b: errors_vs_oracle(batch.fields[b], want[b], samples[b])
                                        for b in range(len(g.blocks))}}
        es = 4 if precision == "split" else 8
        out_bytes = qpts * 22 * es
        in_bytes = sum(b.num_cells * b.element.nodes_per_cell * 4 for b in g.blocks) + g.nodes.numel() * 8
        res[key]["hbm_gbs"] = (out_bytes + in_bytes) / (ms * 1e-3) / 1e9
        del batch
    res["error_sample"] = "16,384 seeded cells per block against the oracle (f64)"
    return res


def extra_hybrid_adjoint():
    """The batched forward + adjoint on the hybrid mesh (2,000,000 Q2 hex, 27 points; 300,000 P2
    prisms, 21; 50,000 P3 tets, 24): seeded standard-normal cotangents on det J and K; one graph
    launch of (a) the double-float forward (f64-accurate x/J/detJ/K) and the split-precision
    adjoint + node sums, (b) the split-precision fused forward + adjoint + node sums, against the
    plain per-block FP64 forward followed by the per-block FP64 adjoint. Bandwidth figures count
    compulsory traffic only (cotangents, fields, dofmaps, nodes, node cotangents)."""
    import torch

    import gridcl_gb300 as tg
    from gridcl_gb300 import meshes, refcell

    mesh = meshes.hybrid_box(2_000_000, 300_000, 50_000)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    rule = tg.QuadRule([tg.PointSet("Hexahedron", *refcell.gauss_rule("Hexahedron", 4)),
                        tg.PointSet("Prism", *refcell.collapsed_rule("Prism", (3, 1, 7))),
                        tg.PointSet("Tetrahedron", *refcell.collapsed_rule("Tetrahedron", (4, 3, 2)))])
    factors = ("points", "jacobian", "detj", "pinv")
    gen = torch.Generator(device="cuda").manual_seed(2026)
    ct64, ct32 = [], []
    qpts = 0
    for blk in g.blocks:
        nq = len(rule.get(blk.element.cell))
        qpts += blk.num_cells * nq
        c = {}
        for name, length in (("detj", 1), ("pinv", 9)):
            f = tg.QuadField.uninit(blk.num_cells, nq, length, 16, torch.float64)
            f.chunks[0].data.normal_(generator=gen)
            c[name] = f
        ct64.append(c)
        ct32.append({k: tg.QuadField([tg.geometry.QuadChunk(0, blk.num_cells, v.chunks[0].data.float())],
                                     blk.num_cells, nq, v.length, 16) for k, v in c.items()})
    for b in range(len(g.blocks)):
        tg.node_incidence(g, b)
    fwd64 = [tg.geometric_factors_block(g, b, rule.get(blk.element.cell), factors) for b, blk in enumerate(g.blocks)]
    locals64 = [torch.empty((blk.num_cells, blk.element.nodes_per_cell, 4), dtype=torch.float64, device="cuda")
                for blk in g.blocks]
    grad64 = torch.zeros((g.nodes.shape[0], 3), dtype=torch.float64, device="cuda")

    def plain():
        grad64.zero_()
        for b, blk in enumerate(g.blocks):
            ps = rule.get(blk.element.cell)
            tg.geometric_factors_block(g, b, ps, factors, out=fwd64[b])
            gb, _ = tg.vjp_block(g, b, ps, ct64[b], local=locals64[b])
            grad64.add_(gb)

    plain()
    plain_ms = event_ms(plain, reps=2, warm=1)
    want = grad64.clone()
    samples = [sample_cells(b.num_cells, 16384, seed=7 + i) for i, b in enumerate(g.blocks)]
    orc_fwd = [oracle_sample(mesh, g, blk.element.cell, blk.element.degree, rule.get(blk.element.cell).points,
                             samples[b], block=b) for b, blk in enumerate(g.blocks)]
    nn = g.nodes.shape[0]

    def compulsory(es_fields: int) -> int:
        """Compulsory traffic of the step: f32 cotangents (det J, K) in, the forward fields out,
        the dofmaps and the nodes in, the node cotangents out."""
        total = nn * 3 * 8 * 2
        for blk in g.blocks:
            nq_b = len(rule.get(blk.element.cell))
            total += blk.num_cells * nq_b * (10 * 4 + 22 * es_fields) + blk.num_cells * blk.element.nodes_per_cell * 4
        return total

    res = {"workload": "hybrid 2,000,000 Q2 hex + 300,000 P2 prisms + 50,000 P3 tets: forward x/J/detJ/K + "
                       "adjoint from detJ and K cotangents + node sums",
           "qpoints": int(qpts),
           "plain_fp64_per_block_fwd_then_vjp": {"ms": plain_ms, "value": qpts / (plain_ms * 1e-3)},
           "error_sample": "forward fields on 16,384 seeded cells per block against the oracle (f64); node "
                           "cotangents against the plain FP64 path's"}
    # two_pass (AdjointBatch's default in split precision): each block's forward on the policy's
    # kernel, its adjoint from the det J and K fields read back (the re-read is not counted as
    # compulsory); the fused pass for comparison.
    for precision, key, es, two in (("df64", "batched_df64_forward_split_adjoint_graph", 8, False),
                                    ("split", "batched_fused_split_graph", 4, False),
                                    ("split", "batched_two_pass_split_graph", 4, True)):
        batch = tg.AdjointBatch(g, rule, ct32, precision=precision, forward=factors, two_pass=two)
        batch.launch()
        ms = event_ms(batch.launch, reps=10)
        alg = compulsory(es)
        res[key] = {"ms": ms, "value": qpts / (ms * 1e-3), "speedup_vs_plain_fp64": plain_ms / ms,
                    "compulsory_bytes": int(alg), "hbm_gbs": alg / (ms * 1e-3) / 1e9,
                    "grad_rel_err_vs_fp64": float((batch.grad - want).abs().max() / want.abs().max()),
                    "forward_error_vs_oracle": {b: errors_vs_oracle(batch.fields[b], orc_fwd[b], samples[b])
                                                for b in range(len(g.blocks))}}
        del batch
        torch.cuda.empty_cache()
    return res


def extra_sphere():
    """Surface TD=2, GD=3: 4,194,304 degree-4 triangles of the refined icosahedron (first cells of
    9 refinements), radius x (1 + 0.02 U), 28-point rule; x, J, area element, normals, K; FP64,
    double-float and split precision, each against the oracle on 65,536 seeded cells."""
    import torch

    import gridcl_gb300 as tg
    from gridcl_gb300 import meshes, refcell

    mesh = meshes.perturbed_radius(meshes.sphere(9, 4, max_cells=4_194_304), 0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    ps = tg.PointSet("Triangle", *refcell.collapsed_rule("Triangle", (7, 4)))
    qpts = mesh.blocks[0].num_cells * len(ps)
    factors = ("points", "jacobian", "detj", "normals", "pinv")
    f64 = tg.geometric_factors_block(g, 0, ps, factors)
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    split = tg.geometric_factors_block(g, 0, ps, factors, precision="split", recomputed=count)
    recomputed = int(count.item())
    ms64 = event_ms(lambda: tg.geometric_factors_block(g, 0, ps, factors, out=f64), reps=3)
    ms32 = event_ms(lambda: tg.geometric_factors_block(g, 0, ps, factors, out=split, precision="split"))
    dfl = tg.geometric_factors_block(g, 0, ps, factors, precision="df64")
    msdf = event_ms(lambda: tg.geometric_factors_block(g, 0, ps, factors, out=dfl, precision="df64"))
    sample = sample_cells(mesh.blocks[0].num_cells)
    want = oracle_sample(mesh, g, "Triangle", 4, ps.points, sample, factors=("x", "j", "detj", "k", "normals"))
    in_bytes = mesh.blocks[0].cells.size * 4 + g.nodes.numel() * 8
    return {"workload": "sphere P4 triangles 4,194,304 cells, 28 pts, x/J/area/normals/K", "qpoints": int(qpts),
            "error_sample": f"{len(sample)} seeded cells against the oracle (f64)",
            "fp64": {"ms": ms64, "value": qpts / (ms64 * 1e-3), "error_vs_oracle": errors_vs_oracle(f64, want, sample)},
            "df64": {"ms": msdf, "value": qpts / (msdf * 1e-3), "speedup_vs_fp64": ms64 / msdf,
                     "hbm_gbs": (qpts * 19 * 8 + in_bytes) / (msdf * 1e-3) / 1e9,
                     "error_vs_oracle": errors_vs_oracle(dfl, want, sample)},
            "split": {"ms": ms32, "value": qpts / (ms32 * 1e-3), "speedup_vs_fp64": ms64 / ms32,
                      "hbm_gbs": (qpts * 19 * 4 + in_bytes) / (ms32 * 1e-3) / 1e9,
                      "fp64_recomputed_points": recomputed,
                      "rel_err_vs_fp64": rel_err_fields(split, f64),
                      "error_vs_oracle": errors_vs_oracle(split, want, sample)}}


def extra_adjoint(n: int = 128, fd_nodes: int = 1000):
    """Forward + adjoint: n^3 Q2 hexahedra, 27-point Gauss, seeded standard-normal cotangents on
    det J and K; the fused split-precision forward + vjp (+ node sums) against the plain FP64
    forward followed by the FP64 vjp; central differences (step 1e-6) at `fd_nodes` seeded nodes (1,000)."""
    import numpy as np
    import torch

    import gridcl_gb300 as tg
    from gridcl_gb300 import meshes, refcell

    mesh = meshes.curved_box("Hexahedron", n, 2, jitter=0.02, seed=2026)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    ps = tg.PointSet("Hexahedron", *refcell.gauss_rule("Hexahedron", 4))
    ncells, nq = mesh.blocks[0].num_cells, len(ps)
    qpts = ncells * nq
    gen = torch.Generator(device="cuda").manual_seed(2026)
    ct64 = {}
    for name, length in (("detj", 1), ("pinv", 9)):
        f = tg.QuadField.uninit(ncells, nq, length, 16, torch.float64)
        f.chunks[0].data.normal_(generator=gen)
        ct64[name] = f
    ct32 = {k: tg.QuadField([tg.geometry.QuadChunk(0, ncells, v.chunks[0].data.float())], ncells, nq,
                            v.length, 16) for k, v in ct64.items()}
    factors = ("points", "jacobian", "detj", "pinv")
    fwd64 = tg.geometric_factors_block(g, 0, ps, factors)
    tg.node_incidence(g, 0)
    local64 = torch.empty((ncells, 27, 4), dtype=torch.float64, device="cuda")
    local32 = torch.empty((ncells, 27, 4), dtype=torch.float32, device="cuda")
    grad64, _ = tg.vjp_block(g, 0, ps, ct64, local=local64)
    grad32, fused = tg.vjp_block(g, 0, ps, ct32, precision="split", forward=factors, local=local32)

    def plain():
        tg.geometric_factors_block(g, 0, ps, factors, out=fwd64)
        tg.vjp_block(g, 0, ps, ct64, local=local64)

    def fused_step():
        tg.vjp_block(g, 0, ps, ct32, precision="split", forward=factors, out=fused, local=local32)

    plain_ms = event_ms(plain, reps=2, warm=1)
    fused_ms = event_ms(fused_step)
    # The two adjoint kernel families on the same step: node rows (four lanes per cell) and sum
    # factorisation (one cell per thread); AUTO picks the latter for Q2 hexahedra.
    families = {}
    for strat in ("direct", "sumfact"):
        with tg.with_strategy(strat):
            ms = event_ms(fused_step)
            ms64 = event_ms(lambda: tg.vjp_block(g, 0, ps, ct64, local=local64), reps=2, warm=1)
            g32, _ = tg.vjp_block(g, 0, ps, ct32, precision="split", forward=factors, local=local32)
            g64, _ = tg.vjp_block(g, 0, ps, ct64, local=local64)
            families[strat] = {"fused_split_ms": ms, "vjp_fp64_ms": ms64,
                               "split_grad_rel_err_vs_fp64": float((g32 - grad64).abs().max() / grad64.abs().max()),
                               "fp64_grad_rel_err": float((g64 - grad64).abs().max() / grad64.abs().max())}
    # Central differences of the FP64 functional at 1,000 seeded nodes against the FP64 adjoint.
    fd = None
    if fd_nodes > 0:
        sample = np.random.default_rng(2026).choice(mesh.num_nodes, fd_nodes, replace=False)
        host = {k: v.to_host_cell_major() for k, v in ct64.items()}
        fd = tg.fd_check(g, 0, ps, {"detj": host["detj"][..., 0], "pinv": host["pinv"]},
                         grad64.cpu().numpy(), sample)
    gerr = float((grad32 - grad64).abs().max() / grad64.abs().max())
    # Two passes: the split forward on the policy's kernel, then the adjoint from the det J and K
    # it wrote (vjp_block(from_fields=...), the tiled kernel).
    fwd32 = tg.geometric_factors_block(g, 0, ps, factors, precision="split")

    def two_pass():
        tg.geometric_factors_block(g, 0, ps, factors, precision="split", out=fwd32)
        tg.vjp_block(g, 0, ps, ct32, precision="split", local=local32, from_fields=fwd32)

    two_ms = event_ms(two_pass)
    grad2, _ = tg.vjp_block(g, 0, ps, ct32, precision="split", local=local32, from_fields=fwd32)
    # The double-float forward (f64-accurate fields) with the split-precision adjoint, one graph.
    dfb = tg.AdjointBatch(g, tg.QuadRule([ps]), [ct32], precision="df64", forward=factors)
    dfb.launch()
    df_ms = event_ms(dfb.launch)
    sample = sample_cells(ncells)
    want = oracle_sample(mesh, g, "Hexahedron", 2, ps.points, sample)

    # Compulsory traffic: f32 cotangents in, the forward fields out, nodes and dofmap in, node
    # cotangents out.
    def compulsory(es_fields):
        return qpts * 10 * 4 + qpts * 22 * es_fields + ncells * 27 * 4 + g.nodes.numel() * 8 * 2

    return {"workload": f"Q2 hex {n}^3, 27 pts, forward (x/J/detJ/K) + adjoint from detJ and K cotangents",
            "qpoints": int(qpts),
            "error_sample": f"forward fields on {len(sample)} seeded cells against the oracle (f64)",
            "plain_fp64_fwd_then_vjp": {"ms": plain_ms, "value": qpts / (plain_ms * 1e-3),
                                        "forward_error_vs_oracle": errors_vs_oracle(fwd64, want, sample)},
            "fused_split_fwd_vjp": {"ms": fused_ms, "value": qpts / (fused_ms * 1e-3),
                                    "speedup_vs_plain_fp64": plain_ms / fused_ms,
                                    "hbm_gbs": compulsory(4) / (fused_ms * 1e-3) / 1e9,
                                    "grad_rel_err_vs_fp64": gerr,
                                    "forward_rel_err_vs_fp64": rel_err_fields(fused, fwd64),
                                    "forward_error_vs_oracle": errors_vs_oracle(fused, want, sample)},
            "two_pass_split_fwd_then_vjp_from_fields": {
                "ms": two_ms, "value": qpts / (two_ms * 1e-3), "speedup_vs_plain_fp64": plain_ms / two_ms,
                "hbm_gbs": compulsory(4) / (two_ms * 1e-3) / 1e9,
                "grad_rel_err_vs_fp64": float((grad2 - grad64).abs().max() / grad64.abs().max())},
            "df64_fwd_split_vjp_graph": {"ms": df_ms, "value": qpts / (df_ms * 1e-3),
                                         "speedup_vs_plain_fp64": plain_ms / df_ms,
                                         "hbm_gbs": compulsory(8) / (df_ms * 1e-3) / 1e9,
                                         "grad_rel_err_vs_fp64": float((dfb.grad - grad64).abs().max() / grad64.abs().max()),
                                         "forward_error_vs_oracle": errors_vs_oracle(dfb.fields[0], want, sample)},
            "families": families,
            "fd_check_fp64": fd}


def extra_pull_back():
    """Pull-back of the 24 quadrature points' images of the 32^3 x 6 curved P2 tetrahedra
    (4.7 M points): the f64 iteration, the FP32 iteration of an f32 mesh, and mixed precision
    (FP32 iteration, three FP64-residual refinements) on the f64 mesh, 16 iterations each."""
    import numpy as np
    import torch

    import gridcl_gb300 as tg

    mesh = build_mesh(32)
    pts, w = rule()
    ps = tg.PointSet("Tetrahedron", pts, w)
    npts = mesh.blocks[0].num_cells * len(pts)
    out = {"workload": "pull-back of the images of 24 points in 32^3x6 curved P2 tetrahedra, 16 iterations",
           "points": int(npts)}
    g64 = tg.Geometry.from_host(mesh, dtype=torch.float64)
    x64 = tg.physical_points_block(g64, 0, ps)
    xi64, st64 = tg.pull_back_block(g64, 0, x64)
    ms = event_ms(lambda: tg.pull_back_block(g64, 0, x64), reps=2, warm=1)
    out["f64"] = {"ms": ms, "value": npts / (ms * 1e-3),
                  "converged": float((st64.to_host_cell_major() <= 1e-13).mean())}
    xs, sts = tg.pull_back_block(g64, 0, x64, precision="split")
    ms_s = event_ms(lambda: tg.pull_back_block(g64, 0, x64, precision="split"))
    d = np.abs(xs.to_host_cell_major() - xi64.to_host_cell_major()).max()
    out["split"] = {"ms": ms_s, "value": npts / (ms_s * 1e-3), "speedup_vs_f64": ms / ms_s,
                    "converged": float((sts.to_host_cell_major() <= 1e-13).mean()),
                    "max_abs_diff_vs_f64": float(d)}
    g32 = tg.Geometry.from_host(mesh, dtype=torch.float32)
    x32 = tg.physical_points_block(g32, 0, ps)
    _, st32 = tg.pull_back_block(g32, 0, x32)
    ms32 = event_ms(lambda: tg.pull_back_block(g32, 0, x32))
    out["f32"] = {"ms": ms32, "value": npts / (ms32 * 1e-3),
                  "converged": float((st32.to_host_cell_major() <= 1e-5).mean())}
    return out


def extra_ordering():
    """Gather locality: the 64^3 x 6 curved P2 tetrahedra with cells and nodes in a seeded random
    order, then reordered along the Hilbert curve of the vertex centroids with nodes numbered by
    first use (host, native); split-precision evaluation of each against the generator's order."""
    import numpy as np
    import torch

    import gridcl_gb300 as tg
    from gridcl_gb300 import meshes

    mesh = build_mesh(64)
    pts, w = rule()
    ps = tg.PointSet("Tetrahedron", pts, w)
    names = ("points", "jacobian", "detj", "pinv")
    mix = meshes.shuffled(mesh, seed=7)
    t0 = time.perf_counter()
    hil, _, _ = meshes.reorder(mix, "hilbert")
    host_s = time.perf_counter() - t0
    out = {"workload": "P2 tet 64^3x6 split evaluation: generator order, shuffled, Hilbert-reordered",
           "hilbert_host_s": host_s}
    for name, m in (("generator", mesh), ("shuffled", mix), ("hilbert", hil)):
        g = tg.Geometry.from_host(m, dtype=torch.float64)
        f = tg.geometric_factors_block(g, 0, ps, names, precision="split")
        out[name + "_ms"] = event_ms(lambda: tg.geometric_factors_block(g, 0, ps, names, out=f, precision="split"))
        del g, f
        torch.cuda.empty_cache()
    return out


def extra_hex_strategies(n: int = 64, cell: str = "Hexahedron"):
    """Curved hexahedra Q1-Q3 (n^3 cells) or prisms P1-P3 (2 n^3 cells) at Gauss rules of 2, 3, 4
    points per direction, evaluated (x/J/detJ/K) under each strategy and precision: ms per launch
    and the kernel family that ran. Run with --workload hex_strategies / prism_strategies (not
    part of the default run)."""
    import numpy as np
    import torch

    import gridcl_gb300 as tg
    from gridcl_gb300 import meshes

    names = ("points", "jacobian", "detj", "pinv")
    label_cells = f"{n}^3 hexahedra" if cell == "Hexahedron" else f"2x{n}^3 prisms"
    out = {"workload": f"curved {label_cells}, degrees 1-3, Gauss rules, x/J/detJ/K"}
    for degree in (1, 2, 3):
        mesh = meshes.curved_box(cell, n, degree, jitter=0.02)
        pts, w = tg.refcell.gauss_rule(cell, 2 * degree)
        ps = tg.PointSet(cell, pts, w)
        for prec, dt in (("split", torch.float64), ("native", torch.float64), ("native", torch.float32)):
            g = tg.Geometry.from_host(mesh, dtype=dt)
            row = {}
            for strat in ("direct", "loops", "sumfact"):
                with tg.with_strategy(strat):
                    f = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
                    fam = tg.last_kernel_family()
                    ms = event_ms(lambda: tg.geometric_factors_block(g, 0, ps, names, out=f, precision=prec),
                                  reps=3, warm=1)
                row[strat] = {"family": fam, "ms": ms}
                del f
            label = "split" if prec == "split" else ("f64" if dt == torch.float64 else "f32")
            out[f"{'Q' if cell == 'Hexahedron' else 'P'}{degree}_{label}"] = row
            del g
            torch.cuda.empty_cache()
    return out


def extra_high_order(n: int = 16, full: bool = True):
    """Curved tetrahedra P4-P6 (6 n^3 cells, 35 / 56 / 84 nodes) at the collapsed Gauss rules of
    degree 2p, x/J/detJ/K: ms per launch and the family that ran, with the stores' bandwidth
    (Q points x 22 f32 outputs). `full`: the loops (global tables), shared (staged tables),
    cooperative and tensor-core kernels and AUTO in split precision, f64 and f32 (run with
    --workload high_order); otherwise (the default run) the tcgen05 and cooperative kernels and AUTO
    in split precision and f32."""
    import torch

    import gridcl_gb300 as tg
    from gridcl_gb300 import meshes

    names = ("points", "jacobian", "detj", "pinv")
    out = {"workload": f"curved tetrahedra P4-P6, 6x{n}^3 cells, Gauss rules of degree 2p, x/J/detJ/K"}
    precisions = ((("split", torch.float64), ("native", torch.float64), ("native", torch.float32)) if full
                  else (("split", torch.float64), ("native", torch.float32)))
    strategies = ("loops", "shared", "cooperative", "tensor", "auto") if full else ("cooperative", "tensor", "auto")
    for degree in (4, 5, 6):
        mesh = meshes.curved_box("Tetrahedron", n, degree, jitter=0.02)
        pts, w = tg.refcell.gauss_rule("Tetrahedron", 2 * degree)
        ps = tg.PointSet("Tetrahedron", pts, w)
        qpts = mesh.blocks[0].num_cells * len(ps)
        for prec, dt in precisions:
            g = tg.Geometry.from_host(mesh, dtype=dt)
            row = {"qpoints": int(qpts)}
            for strat in strategies:
                with tg.with_strategy(strat):
                    f = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
                    fam = tg.last_kernel_family()
                    ms = event_ms(lambda: tg.geometric_factors_block(g, 0, ps, names, out=f, precision=prec),
                                  reps=3, warm=1)
                ob = 8 if (dt == torch.float64 and prec == "native") else 4
                row[strat] = {"family": fam, "ms": ms, "gpts_per_s": qpts / (ms * 1e-3) / 1e9,
                              "store_gbs": qpts * 22 * ob / (ms * 1e-3) / 1e9}
                del f
            if "tensor" in row and "cooperative" in row:
                row["tensor_over_cooperative"] = row["cooperative"]["ms"] / row["tensor"]["ms"]
            label = "split" if prec == "split" else ("f64" if dt == torch.float64 else "f32")
            out[f"P{degree}_{label}"] = row
            del g
            torch.cuda.empty_cache()
    return out


def extra_high_order_case(n: int, degree: int, precision: str):
    """One high-order case for profiling: curved P`degree` tetrahedra 6 n^3, Gauss rule of degree
    2p, x/J/detJ/K under AUTO (the tcgen05 kernel for f32 and split), four launches; the family
    and the last launch's ms."""
    import torch

    import gridcl_gb300 as tg
    from gridcl_gb300 import meshes

    mesh = meshes.curved_box("Tetrahedron", n, degree, jitter=0.02)
    pts, w = tg.refcell.gauss_rule("Tetrahedron", 2 * degree)
    ps = tg.PointSet("Tetrahedron", pts, w)
    g = tg.Geometry.from_host(mesh, dtype=torch.float32 if precision == "f32" else torch.float64)
    prec = "split" if precision == "split" else "native"
    names = ("points", "jacobian", "detj", "pinv")
    f = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
    ms = event_ms(lambda: tg.geometric_factors_block(g, 0, ps, names, out=f, precision=prec), reps=1, warm=2)
    return {"workload": f"curved P{degree} tetrahedra 6x{n}^3, {len(ps)} points, {precision}",
            "family": tg.last_kernel_family(), "ms": ms}


def extra_p1_box():
    """The CPU-runtime workload: 8^3 x 6 = 3,072 P1 tetrahedra, interior nodes jittered by
    +-0.1 h, 14 points (collapsed 7 x 2 x 1); the FP64 and double-float GPU paths, every value held
    against the oracle."""
    import torch

    import gridcl_gb300 as tg
    from gridcl_gb300 import meshes, refcell

    mesh = meshes.curved_box("Tetrahedron", 8, 1, jitter=0.1, amplitude=0.0)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, w = refcell.collapsed_rule("Tetrahedron", (7, 2, 1))
    ps = tg.PointSet("Tetrahedron", pts, w)
    qpts = mesh.blocks[0].num_cells * len(ps)
    every = np.arange(mesh.blocks[0].num_cells)
    want = oracle_sample(mesh, g, "Tetrahedron", 1, pts, every)
    res = {"workload": "P1 tets 8^3x6, 14 pts, f64", "qpoints": int(qpts),
           "error_sample": "every cell and point against the oracle (f64)"}
    for label, prec in (("gpu_fp64", "native"), ("gpu_df64", "df64")):
        out = tg.geometric_factors_block(g, 0, ps, precision=prec)
        ms = event_ms(lambda: tg.geometric_factors_block(g, 0, ps, out=out, precision=prec), reps=20)
        res[label] = {"ms": ms, "value": qpts / (ms * 1e-3), "error_vs_oracle": errors_vs_oracle(out, want, every)}
    return res


# What binds each mode's kernel, from its ncu capture (the profiles of the P2 tetrahedra): the
# double-float and FP64 kernels are bound by an arithmetic pipe, not by HBM.
BINDING = {
    "df64": "FP32 pipes: FMA 54.8 %, ALU 45.5 %, issue 59.9 % of active cycles (ncu, 32^3 x 6 case, monomial form)",
    "f64": "FP64 pipe: 93.7 % of active cycles (ncu)",
    "split": "HBM: stores of the f32 fields (ncu traffic 1.004 x the algorithmic bytes)",
    "f32": "HBM: stores of the f32 fields",
}
# Algorithmic FP64 operations per point of the curved P2 tetrahedra (x: 3 x 10 FMAs, J: 9 x 10
# FMAs, det J and K about 50): the dense direct count; and the FP64 FMA rate measured on this
# GB300 (a dependent-FMA loop over every SM, 1/64 of the FP32 rate).
FLOPS_PER_QPOINT_P2 = 290
FP64_TFLOPS_MEASURED = 1.18


def _roofline(alg: int, ms: float, peaks: dict, traffic, mode: str = "", qpts: int = 0):
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = alg / (ms * 1e-3) / 1e9
    out = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
           "traffic": traffic, "algorithmic_bytes_per_launch": int(alg),
           "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy), of measured" if "hbm_gbs" in peaks
           else "fallback 6800 GB/s"}
    if mode in BINDING:
        out["binding"] = BINDING[mode]
    if mode in ("df64", "f64") and qpts:
        # f64-accurate results per second, in FP64 operations: the double-float path against the
        # FP64 pipe's own peak.
        tf = FLOPS_PER_QPOINT_P2 * qpts / (ms * 1e-3) / 1e12
        out["f64_equivalent"] = {"tflops": tf, "fp64_peak_tflops": FP64_TFLOPS_MEASURED,
                                 "frac_of_fp64_peak": tf / FP64_TFLOPS_MEASURED,
                                 "flops_per_qpoint": FLOPS_PER_QPOINT_P2}
    return out


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
    precision = {"df64": "df64", "split": "split", "f64": "native", "f32": "native"}[args.mode]
    out_es = 4 if args.mode in ("split", "f32") else 8

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
    ms_max = max_over_ranks(ms)
    family = tg.last_kernel_family()

    # The errors against the oracle on a seeded sample of 65,536 cells (the oracle's f64 evaluation
    # of the stored coordinates, as the reference computes it).
    sample = sample_cells(cells)
    want = oracle_sample(mesh, g, "Tetrahedron", 2, pts, sample) if mesh_dtype == torch.float64 else None
    main_err = errors_vs_oracle(out, want, sample) if want is not None else None

    # The plain FP64 GPU path on the same mesh (the metric's baseline), and the other precisions.
    others = {}
    if mesh_dtype == torch.float64:
        for label, prec in (("plain_fp64_gpu", "native"), ("df64_gpu", "df64"), ("split_gpu", "split")):
            if prec == precision:
                continue
            f = tg.geometric_factors_block(g, 0, ps, factors, precision=prec)

            def other_step(f=f, prec=prec):
                tg.geometric_factors_block(g, 0, ps, factors, out=f, precision=prec)

            other_step()
            torch.cuda.synchronize()
            oms = time_steps(other_step, max(3, min(args.steps, 5)), flush, stream)
            others[label] = {"ms_per_step": oms, "value": world * qpts / (oms * 1e-3), "family": tg.last_kernel_family(),
                             "error_vs_oracle": errors_vs_oracle(f, want, sample)}
            if prec == "split":
                es_o = 4
                alg_o = cells * k * 4 + g.nodes.shape[0] * 3 * 8 + qpts * 22 * es_o
                others[label]["roofline"] = {"achieved": alg_o / (oms * 1e-3) / 1e9, "algorithmic_bytes_per_launch": alg_o}
            del f
        torch.cuda.empty_cache()
    plain_ms = ms if precision == "native" and mesh_dtype == torch.float64 else others.get("plain_fp64_gpu", {}).get("ms_per_step")
    recomputed = int(count.item())

    # End to end through the public API, pipelined as a streaming user would run it: every step
    # copies its inputs (nodes and dofmap) from pinned host memory into one of two device input
    # sets on a copy stream, evaluates them on the compute stream, takes the measure (the cell sums
    # of det J * w, then their tree) and copies it back into pinned host memory; the copy of step
    # i + 1 overlaps the evaluation of step i. The timed region ends when the last result has
    # reached the host. The fields stay on the device (the reference's QuadField is
    # device-resident; no field is read back).
    host_nodes = g.nodes.cpu().pin_memory()
    host_dofmap = g.blocks[0].dofmap.cpu().pin_memory()
    h2d = host_nodes.numel() * host_nodes.element_size() + host_dofmap.numel() * 4
    e2e_steps = max(6, min(args.steps, 60))
    geoms = [g, tg.Geometry.from_host(mesh, dtype=mesh_dtype)]
    copy_stream = torch.cuda.Stream()
    comp = torch.cuda.current_stream()
    copied = [torch.cuda.Event() for _ in geoms]
    consumed = [torch.cuda.Event() for _ in geoms]
    results = torch.zeros(e2e_steps, dtype=out["detj"].chunks[0].data.dtype).pin_memory()
    cell_meas = torch.empty(g.blocks[0].num_cells, dtype=results.dtype, device=g.nodes.device)

    def e2e_step(i):
        kk = i % 2
        gk = geoms[kk]
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_event(consumed[kk])  # the evaluation two steps back has read set kk
            gk.nodes.copy_(host_nodes, non_blocking=True)
            gk.blocks[0].dofmap.copy_(host_dofmap, non_blocking=True)
            copied[kk].record(copy_stream)
        comp.wait_event(copied[kk])
        tg.geometric_factors_block(gk, 0, ps, factors, out=out, precision=precision, cell_measure=cell_meas)
        r = tg.measure_block(gk, 0, ps, cell_sums=cell_meas, sync=False)
        consumed[kk].record(comp)
        results[i % e2e_steps].copy_(r[0], non_blocking=True)

    for i in range(4):
        e2e_step(i)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        e2e_step(i)
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) / e2e_steps * 1e3
    vol = float(results[e2e_steps - 1])
    e2e_ms = max_over_ranks(e2e_ms)
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
        dtype = {"df64": "f64", "split": "f32", "f64": "f64", "f32": "f32"}[args.mode]
        traffic = NCU_TRAFFIC_64[args.mode] * qpts / QPOINTS_64 if args.mode in NCU_TRAFFIC_64 else None
        line = {
            "metric": METRIC, "value": whole_job_rate(qpts, world, ms_max), "unit": "qpoints/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": (plain_ms / ms_max) if plain_ms else None,
            "vs_baseline_source": "the plain per-block FP64 GPU path on the same mesh, measured in this run "
                                  "(the metric's baseline; no published number exists for this config)",
            "dtype": dtype,
            "data": "synthetic (seeded sin-mapped, jittered P2 tetrahedral box)",
            "config": {"workload": WORKLOAD, "mode": args.mode, "precision": precision, "mesh_dtype": str(mesh_dtype),
                       "kernel_family": family, "cells": int(cells), "nodes_per_cell": int(k),
                       "nodes": int(g.nodes.shape[0]), "points": int(nq), "qpoints": int(qpts),
                       "outputs_per_qpoint": nout, "output_bytes": out_es, "tile": 16,
                       "l2": "256 MiB flush between steps (outside the timed events); outputs exceed L2",
                       "parallelism": f"replicas x{world}"},
            "error_vs_oracle": main_err,
            "error_sample": f"{len(sample)} seeded cells x {nq} points against the oracle (f64)",
            "roofline": _roofline(alg, ms, peaks, traffic, args.mode, qpts),
            "e2e": {"value": whole_job_rate(qpts, world, e2e_ms), "unit": "qpoints/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": out_es, "ms_per_step": e2e_ms,
                    "measure": vol, "steps": e2e_steps,
                    "pipeline": "host copies of step i+1 overlap the evaluation of step i; fields stay on the device"},
            "gpu_launches": args.steps,
            "clocks": sampler.summary(),
        }
        line.update(others)
        if args.mode == "split":
            line["recomputed_points"] = recomputed
        if not args.no_extras and world == 1:
            workloads = {}
            for name, fn in (("hybrid_batched", extra_hybrid), ("hybrid_forward_adjoint", extra_hybrid_adjoint),
                             ("sphere_surface", extra_sphere),
                             ("q2_forward_adjoint", lambda: extra_adjoint(args.adjoint_n, args.fd_nodes)),
                             ("pull_back", extra_pull_back), ("ordering", extra_ordering),
                             ("p1_box", extra_p1_box), ("high_order", lambda: extra_high_order(args.ho_n, False))):
                try:
                    workloads[name] = fn()
                except Exception as exc:  # reported, not fatal: the main line stands
                    workloads[name] = {"error": f"{type(exc).__name__}: {exc}"}
                torch.cuda.empty_cache()
            line["workloads"] = workloads
        if not args.no_cpu_baseline:
            v, threads, passes = cpu_baseline(mesh, pts)
            line["cpu_baseline"] = {"value": v, "unit": "qpoints/s", "cores": threads, "kind": "port",
                                    "sample": f"{passes} passes over the whole workload (f64), about 10 s"}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


EXTRAS = ("hybrid_batched", "sphere_surface", "q2_forward_adjoint", "pull_back", "ordering", "p1_box",
          "hex_strategies", "prism_strategies", "high_order", "hybrid_forward_adjoint", "high_order_case")


def run_extra(args):
    """One of the other workloads alone (for profiling): its JSON object on one line."""
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    fn = {"hybrid_batched": extra_hybrid, "sphere_surface": extra_sphere,
          "q2_forward_adjoint": lambda: extra_adjoint(args.adjoint_n, args.fd_nodes), "pull_back": extra_pull_back,
          "ordering": extra_ordering, "p1_box": extra_p1_box,
          "hex_strategies": lambda: extra_hex_strategies(args.hex_n),
          "prism_strategies": lambda: extra_hex_strategies(args.hex_n, "Prism"),
          "high_order": lambda: extra_high_order(args.ho_n),
          "high_order_case": lambda: extra_high_order_case(args.ho_n, args.ho_degree, args.ho_precision),
          "hybrid_forward_adjoint": extra_hybrid_adjoint}[args.workload]
    print(json.dumps(fn()), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload != "main":
        run_extra(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
