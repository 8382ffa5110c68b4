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
C++ oracle: the assembly loop + GMRES(100) with the band-100 direct
preconditioner, OpenMP over rows) runs on all host cores at the full size:
one full assembly and one full solve in the set-up, then K timed steps that
each assemble one K-th of the rows, so that the K steps together assemble the
whole matrix again. Both parts are measured at full size; nothing is scaled.
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
        gpu_arm = args.impl == "gb300"
        if gpu_arm:
            torch.cuda.set_device(local)
        # the reference arm runs on the host cores: gloo, no device
        dist.init_process_group("nccl" if gpu_arm else "gloo")
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
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
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


def fp32_peak_tflops():
    """FP32 FMA rate of this GPU from the library's probe (libwbem_peaks.so),
    TFLOP/s, or None."""
    import ctypes as C
    try:
        from wavebem_gb300.build import PEAKS_LIB
        lib = C.CDLL(PEAKS_LIB)
        lib.wbem_peak_probe.restype = C.c_double
        lib.wbem_peak_probe.argtypes = [C.c_int]
        v = lib.wbem_peak_probe(1)
        return v / 1e3 if v > 0 else None
    except OSError:
        return None


def fp64_peak_tflops():
    """FP64 FMA rate of this GPU from the same probe, TFLOP/s, or None."""
    import ctypes as C
    try:
        from wavebem_gb300.build import PEAKS_LIB
        lib = C.CDLL(PEAKS_LIB)
        lib.wbem_peak_probe.restype = C.c_double
        lib.wbem_peak_probe.argtypes = [C.c_int]
        v = lib.wbem_peak_probe(0)
        return v / 1e3 if v > 0 else None
    except OSError:
        return None


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
def config_of(m):
    """The workload description both arms print (the same dict)."""
    return {"workload": f"Wigley tank N={m.n_dofs} mixed-precision assemble+solve",
            "n_dofs": m.n_dofs, "n_cells": m.n_cells, "parallelism": "replicas",
            "solver": "FP32 LU (TF32 tcgen05 trailing updates) + FP64 GMRES refinement",
            "l2": f"inputs larger than L2: the matrices stream {20.0 * m.n_dofs ** 2 / 1e9:.1f} GB "
                  "per assembly (20 N^2 bytes)"}


def oracle_full(m, ptr, idx, b, threads):
    """The reference algorithm on the host cores at the full size: the
    assembly loop (rows over OpenMP threads) and GMRES(100) with the band-100
    direct preconditioner at the reference's tolerance (1e-10, absolute).
    Returns the oracle problem, its solution and the measured times."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle as O
    O.set_threads(threads)
    P = O.Problem(m.X, m.cells, ptr, idx, m.dirichlet)
    t0 = time.perf_counter()
    P.assemble()
    t_asm = time.perf_counter() - t0
    t0 = time.perf_counter()
    phi, dphi, st, its, res = P.solve_system_gmres(b, restart=100, max_steps=3000, tol=1e-10, band=100)
    t_sol = time.perf_counter() - t0
    if st != 0:
        raise RuntimeError(f"oracle GMRES did not converge ({its} its, residual {res})")
    return P, phi, dphi, {"assembly_s": t_asm, "solve_s": t_sol, "gmres_iterations": its,
                          "threads": threads}


def run_reference(args, rank, world):
    """CPU reference arm (rank 0 only): the oracle at the full size on all
    host threads. Set-up: one full assembly and one full solve (measured).
    Timed steps: step k assembles rows [kN/K, (k+1)N/K) of the same matrix,
    so the K timed steps together assemble it once more; their summed time
    plus the measured solve is the value (s per assemble+solve)."""
    if rank != 0:
        return None
    m, ptr, idx, b, hull = workload(args.n)
    threads = os.cpu_count() or 1
    P, _, _, full = oracle_full(m, ptr, idx, b, threads)
    N, K = m.n_dofs, max(1, args.steps)
    bounds = [round(k * N / K) for k in range(K + 1)]
    for k in range(args.warmup):
        P.assemble(rows=(bounds[k % K], bounds[k % K + 1]))
    step_s = []
    for k in range(K):
        t0 = time.perf_counter()
        P.assemble(rows=(bounds[k], bounds[k + 1]))
        step_s.append(time.perf_counter() - t0)
    asm_steps = float(sum(step_s))
    val = asm_steps + full["solve_s"]
    ms_step = 1e3 * asm_steps / K
    sample = (f"full N={N}: assembly measured as the sum of {K} timed row blocks "
              f"({asm_steps:.2f} s; set-up full assembly {full['assembly_s']:.2f} s) + GMRES(100)/"
              f"band-100 solve at tol 1e-10 measured in the set-up ({full['solve_s']:.2f} s, "
              f"{full['gmres_iterations']} its), {threads} threads")
    line = {"metric": METRIC, "value": val, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": K, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic Wigley towing-tank mesh (seeded)",
            "config": config_of(m),
            "step": f"assembly of 1/{K} of the rows of the N={N} matrix (all panels), "
                    f"{threads} host threads",
            "measured": {"assembly_steps_s": asm_steps, "assembly_setup_s": full["assembly_s"],
                         "solve_s": full["solve_s"], "gmres_iterations": full["gmres_iterations"],
                         "step_s": step_s},
            "modelled": None,
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return line


# ------------------------------------------------------------------ GPU side
# DRAM traffic of one launch of the roofline kernels (dram__bytes_read.sum +
# dram__bytes_write.sum) from one ncu capture each at N = 8,192. All three
# move O(N^2) bytes per launch, so a launch at N dofs is scaled by
# (N / 8192)^2.
NCU_TRAFFIC = {
    "k_tile_mixed": 17.5424e6 + 1314.548e6,
    "k_matvec_mixed": 537.038080e6 + 3.272192e6,
    "k_trsv_wave": 136.424192e6 + 3.058176e6,
}


# Warp instructions of one far-field assembly launch at N = 8,192 (ncu
# smsp__inst_executed.sum); they scale with the (row, panel) pairs, i.e. with
# N^2 on the same family of meshes.
NCU_TILE_INSTR = 2949815885.0

# DRAM bytes of a trailing-update launch over its algorithmic C traffic
# (8 bytes per element of C, read and written once): 2.205 GB against
# 1.887 GB for the largest launch at N = 16,384 (15,360 x 15,360, K = 512,
# TF32), from one ncu capture; the operands add the rest.
NCU_GEMM_TRAFFIC_RATIO = (1.309495e9 + 0.895142e9) / (8.0 * 15360 * 15360)


def ncu_traffic(kernel, n):
    """(bytes per launch at n dofs, how it was obtained) or (None, None)."""
    t = NCU_TRAFFIC.get(kernel)
    if t is None:
        return None, None
    return t * (n / 8192.0) ** 2, "ncu capture at N = 8192, scaled by (N / 8192)^2"


class KernelProfile:
    """wbem_kernel_profile (include/wbem_kernels.h)."""

    @staticmethod
    def struct():
        import ctypes as C

        class P(C.Structure):
            _fields_ = [("gemm_ms", C.c_double), ("gemm_flop", C.c_double), ("gemm_launches", C.c_int),
                        ("diag_ms", C.c_double), ("diag_launches", C.c_int),
                        ("panel_ms", C.c_double), ("panel_launches", C.c_int),
                        ("matvec_ms", C.c_double), ("matvec_bytes", C.c_double),
                        ("matvec_launches", C.c_int),
                        ("trsv_ms", C.c_double), ("trsv_bytes", C.c_double), ("trsv_launches", C.c_int),
                        ("reserved", C.c_int * 8)]
        return P


def timed(stream, fn, reps):
    import torch
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        t0.record(stream)
        for _ in range(reps):
            fn()
        t1.record(stream)
    torch.cuda.synchronize()
    return t0.elapsed_time(t1) / reps / 1e3


def run_gpu(args, rank, world, local):
    import ctypes
    import torch
    from wavebem_gb300 import meshes as M
    from wavebem_gb300.bem_problem import (METHOD_FMA, PREC_FP64, PREC_MIXED, SOLVER_GMRES_IR,
                                           SOLVER_LU, BEMProblem, load_library)

    torch.cuda.set_device(local)
    L = load_library()
    L.wbem_set_stream.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.wbem_set_profiling.argtypes = [ctypes.c_void_p, ctypes.c_int]
    Prof = KernelProfile.struct()
    L.wbem_get_kernel_profile.argtypes = [ctypes.c_void_p, ctypes.POINTER(Prof)]
    m, ptr, idx, b, hull = workload(args.n)
    N = m.n_dofs
    stream = torch.cuda.Stream()

    def problem(prec, mesh=None, p=None, i=None):
        mesh = m if mesh is None else mesh
        g = BEMProblem(mesh.X, mesh.cells, mesh.dirichlet, ptr if p is None else p,
                       idx if i is None else i, device=local, precision=prec)
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

    # adjoint of the hull force on the same assembly (LU factors reused)
    g.solve(phi, dphi, b)
    adj_s = timed(stream, lambda: g.force_adjoint(hull, b), 2)
    adjoint = {"s": adj_s, "n_dofs": N, "over_forward": adj_s / (ms_step / 1e3),
               "what": "dF_x/dX (all nodes) and dF_x/dtmp_rhs after one mixed assemble+solve"}

    # instrumented pass: kernel classes bracketed by events (serialised factor)
    L.wbem_set_profiling(g.h, 1)
    g.solve(phi, dphi, b)
    pr = Prof()
    assert L.wbem_get_kernel_profile(g.h, ctypes.byref(pr)) == 0
    L.wbem_set_profiling(g.h, 0)
    st_prof = g.stats()
    kprof = {k: getattr(pr, k) for k, _ in Prof._fields_ if k != "reserved"}
    kprof["tile_ms"] = st_prof["t_assemble_ms"]
    kprof["factor_ms_serialised"] = st_prof["t_factor_ms"]

    # the refinement solver variant on the same workload
    variants = {}
    ir_s = timed(stream, lambda: g.solve(phi, dphi, b, solver=SOLVER_GMRES_IR), 2)
    st_ir = g.stats()
    phi_ir, dphi_ir = phi.copy(), dphi.copy()
    variants["gmres_ir"] = {"s": ir_s, "iterations": st_ir["iterations"],
                            "outer_iterations": st_ir["outer_iterations"],
                            "what": "FP64 refinement over inner block-Jacobi GMRES on the FP32 "
                                    "system matrix (no LU)"}
    g.close()
    del g

    # the FMA method on the same workload (O(N) memory and mat-vec), and on a
    # 135,002-node cube-sphere whose dense N and D would need 290 GB
    gf = BEMProblem(m.X, m.cells, m.dirichlet, ptr, idx, device=local, method=METHOD_FMA, fma_order=6)
    assert L.wbem_set_stream(gf.h, ctypes.c_void_p(stream.cuda_stream)) == 0
    phi_f, dphi_f = b.copy(), b.copy()
    gf.solve(phi_f, dphi_f, b)
    tree_f = gf.stats()["t_assemble_ms"]  # octree and lists, built by the first solve only
    fma_s = timed(stream, lambda: gf.solve(phi_f, dphi_f, b), 2)
    st_f = gf.stats()
    F_f = gf.hull_force(hull, phi_f, dphi_f)
    vm_s = timed(stream, lambda: gf.vmult(b), 5)
    variants["fma"] = {"s": fma_s, "order": 6, "iterations": st_f["iterations"],
                       "assemble_ms": st_f["t_geometry_ms"] + st_f["t_singular_ms"] + st_f["t_alpha_ms"],
                       "tree_build_ms": tree_f,
                       "vmult_ms_host": vm_s * 1e3,
                       "what": "octree + Chebyshev far field (order 6) + on-the-fly near field with FP64 "
                               "close-pair corrections, FP64 GMRES with near-field block-Jacobi"}
    gf.close()
    del gf
    ms_ = M.cube_sphere_mesh(150)
    ps_, is_ = M.double_nodes(ms_.X, ms_.cells)
    p_s, dp_s = M.sphere_harmonics(ms_.X, seed=1)
    for order in (6, 8):
        gs = BEMProblem(ms_.X, ms_.cells, ms_.dirichlet, ps_, is_, device=local, method=METHOD_FMA,
                        fma_order=order, max_steps=2000)
        assert L.wbem_set_stream(gs.h, ctypes.c_void_p(stream.cuda_stream)) == 0
        ph_s, dph_s = p_s.copy(), np.zeros_like(p_s)
        gs.solve(ph_s, dph_s, p_s)
        tree_s = gs.stats()["t_assemble_ms"]
        s_s = timed(stream, lambda: gs.solve(ph_s, dph_s, p_s), 1)
        variants[f"fma_sphere_order{order}"] = {
            "s": s_s, "n_dofs": ms_.n_dofs, "iterations": gs.stats()["iterations"],
            "tree_build_ms": tree_s,
            "rel_err_vs_exact": float(np.linalg.norm(dph_s - dp_s) / np.linalg.norm(dp_s)),
            "what": "all-Dirichlet cube-sphere (harmonic polynomial data), dphi/dn against the exact one"}
        gs.close()
        del gs

    # shape-parameter adjoint workload: N = 8,192 Wigley hull with 8 seeded
    # shape parameters (the configuration's seeds)
    m8, p8, i8, b8 = M.config_case("c3")
    h8 = np.nonzero(m8.face == M.HULL)[0].astype(np.int32)
    g8 = problem(PREC_MIXED, m8, p8, i8)
    ph8, dp8 = b8.copy(), b8.copy()
    g8.solve(ph8, dp8, b8)
    f8 = timed(stream, lambda: g8.solve(ph8, dp8, b8), 2)
    a8 = timed(stream, lambda: g8.force_adjoint(h8, b8), 2)
    adjoint["n8192"] = {"forward_s": f8, "adjoint_s": a8, "over_forward": a8 / f8}
    g8.close()
    del g8

    extra = {}
    nrm = lambda a, r: float(np.linalg.norm(a - r) / np.linalg.norm(r))
    fp64 = None
    if not args.no_fp64:
        g64 = problem(PREC_FP64)
        p64, d64 = b.copy(), b.copy()
        g64.solve(p64, d64, b)  # warm-up
        fp64_s = timed(stream, lambda: g64.solve(p64, d64, b), 2)
        st64 = g64.stats()
        F64 = g64.hull_force(hull, p64, d64)
        fp64 = (p64, d64, F64)
        extra = {"fp64_gpu_s": fp64_s, "speedup_vs_fp64_gpu": fp64_s / (ms_step / 1e3),
                 "fp64_gmres_iterations": st64["iterations"],
                 "rel_err_vs_fp64": {"phi": nrm(phi_mx, p64), "dphi_dn": nrm(dphi_mx, d64),
                                     "hull_force": abs(F_mx - F64) / abs(F64)},
                 "fp64_phases_ms": {k: st64[k] for k in phase}}
        variants["gmres_ir"]["rel_err_vs_fp64"] = {"phi": nrm(phi_ir, p64), "dphi_dn": nrm(dphi_ir, d64)}
        variants["fma"]["rel_err_vs_fp64"] = {"phi": nrm(phi_f, p64), "dphi_dn": nrm(dphi_f, d64),
                                              "hull_force": abs(F_f - F64) / abs(F64)}
        g64.close()
        del g64

    peaks = load_peaks()
    out = None
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            # the reference algorithm at the full size on every host thread:
            # the CPU baseline, and the checker of every output of both GPU forms
            threads = os.cpu_count() or 1
            P, phi_o, dphi_o, full = oracle_full(m, ptr, idx, b, threads)
            F_o = P.hull_force(m.cells[hull], phi_o, dphi_o)
            del P
            v = full["assembly_s"] + full["solve_s"]
            cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"the whole workload, measured once: assembly {full['assembly_s']:.2f} s + "
                             f"GMRES(100)/band-100 solve at tol 1e-10 {full['solve_s']:.2f} s "
                             f"({full['gmres_iterations']} its) on {threads} host threads"}
            errs = {"mixed": {"phi": nrm(phi_mx, phi_o), "dphi_dn": nrm(dphi_mx, dphi_o),
                              "hull_force": abs(F_mx - F_o) / abs(F_o)},
                    "gmres_ir": {"phi": nrm(phi_ir, phi_o), "dphi_dn": nrm(dphi_ir, dphi_o)},
                    "fma": {"phi": nrm(phi_f, phi_o), "dphi_dn": nrm(dphi_f, dphi_o),
                            "hull_force": abs(F_f - F_o) / abs(F_o)}}
            if fp64 is not None:
                errs["fp64"] = {"phi": nrm(fp64[0], phi_o), "dphi_dn": nrm(fp64[1], dphi_o),
                                "hull_force": abs(fp64[2] - F_o) / abs(F_o)}
            extra["rel_err_vs_oracle"] = errs
            extra["oracle_note"] = ("oracle = the reference algorithm restated in FP64 (C++), its GMRES "
                                    "at the reference's tolerance 1e-10 (converged to ~1e-11 relative)")
        hbm = peaks.get("hbm_gbs")
        tc = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))
        src = "of fallback" if peaks.get("fallback") else "of measured"
        fp32 = fp32_peak_tflops()
        fp64_peak = fp64_peak_tflops()
        # every kernel class with its own bound; the dominant one is the roofline
        kernels = []
        if kprof["gemm_ms"] > 0:
            a = kprof["gemm_flop"] / (kprof["gemm_ms"] / 1e3) / 1e12
            # one TF32 product per trailing update; its dense rate is half the
            # BF16 rate (nominal 1.1 vs 2.25 PFLOP/s), applied to the measured
            # sustained BF16 figure
            tf32 = tc / 2.0
            # sum of M x Nc over the launches (every trailing update has K = 512)
            mn = kprof["gemm_flop"] / (2.0 * 512)
            kernels.append({"kernel": "k_gemm_tc<tf32>", "bound": "tensor", "ms": kprof["gemm_ms"],
                            "launches": kprof["gemm_launches"], "achieved": a, "peak": tf32,
                            "unit": "TFLOP/s", "frac": a / tf32,
                            "work": "2 M N K per launch (one TF32 product per trailing update)",
                            "peak_source": f"half of MEASURED_PEAKS.json bf16_tflops_sustained ({src}): "
                                           "the TF32 dense rate",
                            "traffic_per_launch": NCU_GEMM_TRAFFIC_RATIO * 8.0 * mn / kprof["gemm_launches"],
                            "traffic_source": "8 bytes per C element per launch (the average launch) times "
                                              "the DRAM / C-traffic ratio of one ncu capture at N = 16384"})
        # the far-field assembly: bound by FP32 arithmetic (work counted as 36
        # flop per regular kernel evaluation, 16 evaluations per (row, panel)
        # pair); its HBM figure is reported beside it
        tile_s = kprof["tile_ms"] / 1e3
        tile = {"kernel": "k_tile_mixed", "ms": kprof["tile_ms"], "launches": 1}
        t_flop = 36.0 * 16.0 * N * m.n_cells
        if fp32:
            a = t_flop / tile_s / 1e12
            tile.update({"bound": "fp32", "achieved": a, "peak": fp32, "unit": "TFLOP/s", "frac": a / fp32,
                         "work": "36 flop per regular kernel evaluation x 16 N C (the plain evaluation count; "
                                 "the double-float panel term and the column-tile redundancy are not counted)",
                         "peak_source": "FP32 FMA loop (wbem_peak_probe) on this GPU, measured in this run"})
        a = 20.0 * N * N / tile_s / 1e9
        tile["hbm"] = {"achieved": a, "peak": hbm, "unit": "GB/s", "frac": a / hbm,
                       "work": "N and D as (hi, lo) float pairs and the FP32 system copy: 20 N^2 bytes",
                       "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({src})"}
        if "bound" not in tile:
            tile.update({"bound": "hbm", **{k: tile["hbm"][k] for k in ("achieved", "peak", "unit", "frac",
                                                                        "work", "peak_source")}})
        sm_mhz = (clk or {}).get("sm_mhz")
        if sm_mhz:
            # instruction issue: 4 warp instructions per SM per clock at most
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            ins = NCU_TILE_INSTR * (N / 8192.0) ** 2 / tile_s
            pk = 4.0 * sms * sm_mhz * 1e6
            tile["issue_roof"] = {
                "achieved": ins / 1e12, "peak": pk / 1e12, "unit": "T warp-instr/s", "frac": ins / pk,
                "work": "warp instructions of one launch from an ncu capture at N = 8,192, scaled by (N / 8192)^2",
                "peak_source": "4 per SM per clock at the median SM clock sampled during the timed region"}
        kernels.append(tile)
        if kprof["matvec_ms"] > 0:
            a = kprof["matvec_bytes"] / (kprof["matvec_ms"] / 1e3) / 1e9
            kernels.append({"kernel": "k_matvec_mixed", "bound": "hbm", "ms": kprof["matvec_ms"],
                            "launches": kprof["matvec_launches"], "achieved": a, "peak": hbm,
                            "unit": "GB/s", "frac": a / hbm, "work": "8 N^2 bytes per launch",
                            "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({src})"})
        if kprof["trsv_ms"] > 0:
            a = kprof["trsv_bytes"] / (kprof["trsv_ms"] / 1e3) / 1e9
            kernels.append({"kernel": "k_trsv_wave", "bound": "hbm", "ms": kprof["trsv_ms"],
                            "launches": kprof["trsv_launches"], "achieved": a, "peak": hbm,
                            "unit": "GB/s", "frac": a / hbm, "work": "2 N^2 bytes per sweep",
                            "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({src})"})
        kernels.append({"kernel": "k_diag_block", "ms": kprof["diag_ms"], "launches": kprof["diag_launches"]})
        kernels.append({"kernel": "k_panel_small", "ms": kprof["panel_ms"],
                        "launches": kprof["panel_launches"]})
        for k in kernels:
            tb, ts = ncu_traffic(k["kernel"], N)
            if tb is not None:
                k["traffic_per_launch"] = tb
                k["traffic_source"] = ts
        if "fp64_phases_ms" in extra and fp64_peak:
            # the plain FP64 form's far-field assembly against the FP64 FMA rate:
            # ~30 FP64 flop per regular evaluation, 16 N C evaluations
            t64 = extra["fp64_phases_ms"]["t_assemble_ms"] / 1e3
            a = 30.0 * 16.0 * N * m.n_cells / t64 / 1e12
            extra["fp64_assembly_roof"] = {
                "kernel": "k_tile_fp64", "bound": "fp64", "achieved": a, "peak": fp64_peak,
                "unit": "TFLOP/s", "frac": a / fp64_peak,
                "work": "30 FP64 flop per regular kernel evaluation x 16 N C (column-tile redundancy not counted)",
                "peak_source": "FP64 FMA loop (wbem_peak_probe) on this GPU, measured in this run"}
        dom = max((k for k in kernels if "bound" in k), key=lambda k: k["ms"])
        per_launch = dom["ms"] / max(1, dom["launches"])
        roof = {"bound": dom["bound"], "kernel": dom["kernel"], "achieved": dom["achieved"],
                "peak": dom["peak"], "unit": dom["unit"], "frac": dom["frac"],
                "traffic": dom.get("traffic_per_launch"),
                "traffic_source": dom.get("traffic_source"), "ms_per_launch": per_launch,
                "peak_source": dom["peak_source"],
                "timing": "CUDA events around each launch on its own stream, in an instrumented "
                          "pass after the timed region (factorisation serialised on one stream)"}
        if "hbm" in dom:
            roof["hbm"] = dom["hbm"]
        if "issue_roof" in dom:
            roof["issue_roof"] = dom["issue_roof"]
        out = {"metric": METRIC, "value": ms_step / 1e3, "unit": UNIT, "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
               "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32+f64 (mixed)", "data": "synthetic Wigley towing-tank mesh (seeded)",
               "config": config_of(m),
               "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(N * 3 * 8 + N * 8),
                       "d2h_bytes_per_step": int(N * 8)},
               "gpu_launches": int(launches),
               "phases_ms": per_phase, "gmres_iterations": iters,
               "roofline": roof, "kernels": kernels, "adjoint": adjoint, "variants": variants,
               "cpu_baseline": cpu, "clocks": clk}
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
