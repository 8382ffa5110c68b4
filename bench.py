"""Benchmark of the GB300 collocation-BEM hot path.

Headline workload: the Wigley towing tank refined to N = 32,768 dofs (32,768
nodes, Q1 panels, double nodes on the patch edges), mixed Dirichlet (free
surface) / Neumann (hull, bottom, walls) data, one step = assemble_system +
solve_system in the mixed-precision form (double-float panel base + FP32
point differences for the far field, FP64 near/singular field and alpha,
FP32 LU with BF16x3 tcgen05 trailing updates, FP64 GMRES refinement).
Metric: seconds per assemble+solve (lower is better). The plain FP64 GPU form
and the adjoint are measured on the same mesh and reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--n 32768] [--impl reference]

With --impl reference the reference algorithm's CPU implementation (the
C++ oracle: serial assembly loop + GMRES(100) with the band-100 direct
preconditioner) is timed on the host cores on a bounded sample of the same
workload and scaled to the full size.
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

METRIC = "assemble+solve s at N=32k: mixed-prec vs FP64 GPU at 1e-8 rel err; adjoint s"
UNIT = "s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--n", type=int, default=32768)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison run")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    return p.parse_args()


def dist_init(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampler over the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
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
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "fallback": True}


def workload(n):
    from wavebem_gb300 import meshes as M
    m = M.wigley_mesh(n)
    ptr, idx = M.double_nodes(m.X, m.cells)
    b = M.wigley_bc(m, seed=2)
    hull = np.nonzero(m.face == M.HULL)[0].astype(np.int32)
    return m, ptr, idx, b, hull


# ------------------------------------------------------------------ CPU side
def cpu_sample(m, ptr, idx, threads: int, budget_rows: int):
    """Reference algorithm on the host: serial-loop assembly of a row sample
    (scaled to all N rows) + GMRES(100)/band-100 solve measured on the
    2,000-dof Wigley case and scaled by (N/2000)^2 (its cost is the O(N^2)
    mat-vecs). Returns (seconds per assemble+solve at N, description)."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle as O
    from wavebem_gb300 import meshes as M
    N = m.n_dofs
    P = O.Problem(m.X, m.cells, ptr, idx, m.dirichlet)
    rows = min(N, budget_rows)
    t0 = time.perf_counter()
    P.assemble(rows=(0, rows))
    t_asm = (time.perf_counter() - t0) * N / rows
    ms = M.wigley_mesh(2000)
    ps, pi = M.double_nodes(ms.X, ms.cells)
    Ps = O.Problem(ms.X, ms.cells, ps, pi, ms.dirichlet)
    Ps.assemble()
    bs = M.wigley_bc(ms, seed=2)
    t0 = time.perf_counter()
    _, _, st, its, res = Ps.solve_system_gmres(bs, restart=100, max_steps=1000, tol=1e-10, band=100)
    t_sol = (time.perf_counter() - t0) * (N / ms.n_dofs) ** 2
    desc = (f"assembly of rows 0..{rows} of {N} (all {m.n_cells} panels) scaled x{N / rows:.0f}; "
            f"GMRES(100)+band-100 solve of the 2,000-dof case ({its} its) scaled by (N/2000)^2")
    return t_asm + t_sol, desc, t_asm, t_sol


def run_reference(args, rank, world):
    if rank != 0:
        return
    m, ptr, idx, b, hull = workload(args.n)
    threads = os.cpu_count() or 1
    times = []
    for k in range(args.warmup + args.steps):
        v, desc, ta, ts = cpu_sample(m, ptr, idx, threads, budget_rows=8 * threads)
        if k >= args.warmup:
            times.append(v)
    val = float(np.median(times))
    line = {"metric": METRIC, "value": val, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": val * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic Wigley towing-tank mesh (seeded)",
            "config": {"workload": f"Wigley tank N={m.n_dofs} assemble+solve (CPU oracle, all host threads)",
                       "n_dofs": m.n_dofs, "n_cells": m.n_cells},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU side
def run_gpu(args, rank, world, local):
    import ctypes
    import torch
    from wavebem_gb300.bem_problem import PREC_FP64, PREC_MIXED, BEMProblem, load_library

    torch.cuda.set_device(local)
    L = load_library()
    L.wbem_set_stream.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    m, ptr, idx, b, hull = workload(args.n)
    N = m.n_dofs
    stream = torch.cuda.Stream()

    def problem(prec):
        g = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, device=local, precision=prec)
        assert L.wbem_set_stream(g.h, ctypes.c_void_p(stream.cuda_stream)) == 0
        return g

    g = problem(PREC_MIXED)
    phi = b.copy()
    dphi = b.copy()
    # warm-up
    for _ in range(args.warmup):
        g.solve(phi, dphi, b)
    torch.cuda.synchronize()
    # timed: device-resident inputs (geometry already on the GPU): assemble + solve_system
    clocks = Clocks(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    phase = {k: 0.0 for k in ("t_geometry_ms", "t_assemble_ms", "t_singular_ms", "t_alpha_ms",
                              "t_system_ms", "t_factor_ms", "t_solve_ms")}
    launches = 0
    iters = []
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(args.steps):
            g.solve(phi, dphi, b)
            st = g.stats()
            for k in phase:
                phase[k] += st[k]
            launches += st["kernel_launches"]
            iters.append(st["iterations"])
        ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms_step = ev0.elapsed_time(ev1) / args.steps
    ms_step = allmax(world, ms_step)
    phi_mx, dphi_mx = phi.copy(), dphi.copy()
    F_mx = g.hull_force(hull, phi_mx, dphi_mx)
    # end to end through the C ABI with host buffers: new support points (H2D),
    # tmp_rhs (H2D), phi / dphi_dn back (D2H)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        g.update_nodes(m.X)
        g.solve(phi, dphi, b)
    torch.cuda.synchronize()
    e2e = allmax(world, (time.perf_counter() - t0) / args.steps)
    per_phase = {k: v / args.steps for k, v in phase.items()}
    g.close()
    del g

    extra = {}
    if not args.no_fp64:
        g64 = problem(PREC_FP64)
        p64, d64 = b.copy(), b.copy()
        g64.solve(p64, d64, b)  # warm-up
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        reps = 2
        with torch.cuda.stream(stream):
            t0.record(stream)
            for _ in range(reps):
                g64.solve(p64, d64, b)
            t1.record(stream)
        torch.cuda.synchronize()
        st64 = g64.stats()
        fp64_s = t0.elapsed_time(t1) / reps / 1e3
        F64 = g64.hull_force(hull, p64, d64)
        nrm = lambda a, r: float(np.linalg.norm(a - r) / np.linalg.norm(r))
        extra = {"fp64_gpu_s": fp64_s, "speedup_vs_fp64_gpu": fp64_s / (ms_step / 1e3),
                 "fp64_gmres_iterations": st64["iterations"],
                 "rel_err_vs_fp64": {"phi": nrm(phi_mx, p64), "dphi_dn": nrm(dphi_mx, d64),
                                     "hull_force": abs(F_mx - F64) / abs(F64)},
                 "fp64_phases_ms": {k: st64[k] for k in phase}}
        g64.close()
        del g64

    peaks = load_peaks()
    out = None
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            v, desc, ta, ts = cpu_sample(m, ptr, idx, 1, budget_rows=16)
            cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "sample": desc}
        asm_ms = per_phase["t_assemble_ms"]
        fac_ms = per_phase["t_factor_ms"]
        # roofline of the dominant kernel
        nblk = (N + 127) // 128
        gemm_flop = sum(3 * 2.0 * (N - (k + 1) * 128) ** 2 * 128 for k in range(nblk) if N - (k + 1) * 128 > 0)
        if fac_ms >= asm_ms:
            achieved = gemm_flop / (fac_ms / 1e3) / 1e12
            roof = {"bound": "tensor", "kernel": "LU (BF16x3 tcgen05 trailing updates + panels)",
                    "achieved": achieved, "peak": peaks.get("bf16_tflops"), "unit": "TFLOP/s",
                    "frac": achieved / peaks.get("bf16_tflops"), "traffic": None,
                    "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst) — of measured"}
        else:
            bytes_ = 2 * N * N * 8.0  # N and D as (hi, lo) float pairs
            achieved = bytes_ / (asm_ms / 1e3) / 1e9
            roof = {"bound": "hbm", "kernel": "k_tile_mixed (assembly)", "achieved": achieved,
                    "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                    "frac": achieved / peaks.get("hbm_gbs"), "traffic": None,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs — of measured; the kernel is FP32-ALU bound"}
        out = {"metric": METRIC, "value": ms_step / 1e3, "unit": UNIT, "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
               "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32+f64 (mixed)", "data": "synthetic Wigley towing-tank mesh (seeded)",
               "config": {"workload": f"Wigley tank N={N} mixed-precision assemble+solve",
                          "n_dofs": N, "n_cells": m.n_cells, "parallelism": "replicas",
                          "l2": "inputs (N, D: 17 GB) larger than L2"},
               "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(N * 3 * 8 + N * 8),
                       "d2h_bytes_per_step": int(N * 8)},
               "gpu_launches": int(launches),
               "phases_ms": per_phase, "gmres_iterations": iters,
               "roofline": roof, "cpu_baseline": cpu, "clocks": clk}
        out.update(extra)
        print(json.dumps(out), flush=True)
    return out


def main():
    args = parse()
    rank, world, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
