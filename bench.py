#!/usr/bin/env python3
"""Newton-step benchmark of the GB300 backend for feNG's assembly + Krylov hot path.

Workload (one GPU): steady incompressible Navier-Stokes, Kovasznay flow at
Re = 40 on [-0.5, 1.5]^2, 256 x 256 cells split into 2 triangles each
(131,072 P2-P1 Taylor-Hood triangles, 588,290 unknowns), interior vertices
jittered by +-0.1 h (SplitMix64, seed 1), velocity Dirichlet on "Bord",
pressure fixed at "PointPression", quadrature of degree 8.

A step = one full Newton solve from the boundary-initialised zero state to
||R||_inf / ||R_0||_inf <= 1e-8 (R assembled in FP64):
  * plain FP64: FP64 Jacobian, FP64 FGMRES(50) at the reference's linear
    tolerance 1e-8 (feLinearSystem::_rel_tol);
  * mixed (the headline `value`): FP32 Jacobian, FP32 SpMV, multigrid
    preconditioner and Arnoldi basis inside FGMRES (FP64 Hessenberg, FP64
    restart residuals), inexact Newton (linear tolerance
    max(1e-6, min(1e-2, 0.1 ||R||/||R0||))).
The learned initial guess applies to transient runs (time history); this
steady workload has none, so its mixed arm runs without it.  The
`transient` object times configuration C4 (lid-driven cavity, Re 1000,
384 x 384, BDF2 dt 0.005, 40 steps from rest): plain FP64 with the
reference's guess against mixed with the extrapolated and the learned guess.

Output: one JSON line (see the repository's benchmark contract).  With
``--impl reference`` the CPU oracle (a restatement of the reference's CPU
algorithms, OpenMP on all host cores) is timed on a bounded sample instead.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

RE = 40.0
METRIC = "newton_step_s"
UNIT = "s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256, help="cells per side")
    ap.add_argument("--transient-steps", type=int, default=40,
                    help="BDF2 steps of the lid-driven cavity leg (configuration C4)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier / max over ranks (replicas only: no data-path collective)."""

    def __init__(self, ws):
        self.ws = ws
        self.pg = None
        if ws > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t)
        return float(t.item())


def build_problem(n):
    from feng_gb300 import kovasznay
    return kovasznay.build(n, RE)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(device)], stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait(timeout=10)
        self.f.flush()
        rows = [l.split(",") for l in Path(self.f.name).read_text().splitlines() if l.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) >= 9 for i in range(4)
                          if r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def make_system(num, forms, precision):
    from feng_gb300 import kovasznay
    return kovasznay.make_system(num, forms, precision)


def newton_opts(precision):
    from feng_gb300 import kovasznay
    return kovasznay.newton_options(precision)


def run_newton(sys_, nl):
    import feng_gb300 as fe
    return fe.solveNewtonRaphson(sys_, None, nl)


def timed_steps(sys_, nl, steps, warmup, dist):
    """K Newton solves from the saved initial state, device-timed with CUDA events."""
    from feng_gb300._lib import check
    lib = sys_.lib
    check(lib.fe_cuda_save_solution(sys_._h))
    for _ in range(warmup):
        check(lib.fe_cuda_restore_solution(sys_._h))
        st = run_newton(sys_, nl)
    sys_.synchronize()
    dist.barrier()
    sys_.synchronize()
    stats = []
    l0 = C.c_int64()
    check(lib.fe_cuda_launch_count(C.byref(l0)))
    sys_.resetTimes()
    check(lib.fe_cuda_event_record(sys_._h, 0))
    for _ in range(steps):
        check(lib.fe_cuda_restore_solution(sys_._h))
        stats.append(run_newton(sys_, nl))
    check(lib.fe_cuda_event_record(sys_._h, 1))
    ms = C.c_double()
    check(lib.fe_cuda_event_elapsed(sys_._h, 0, 1, C.byref(ms)))
    sys_.synchronize()
    dist.barrier()
    l1 = C.c_int64()
    check(lib.fe_cuda_launch_count(C.byref(l1)))
    return ms.value / 1e3, stats, l1.value - l0.value, sys_.times()


def e2e_steps(sys_, nl, steps):
    """Same metric through the public API with host buffers: every step
    uploads the initial state from pinned host memory, runs the Newton solve
    and reads the solution back into pinned host memory."""
    import torch
    import feng_gb300 as fe
    from feng_gb300._lib import check
    lib = sys_.lib
    # The initial state saved before the timed device steps (with its
    # boundary values), fetched to the host outside the timed region.
    check(lib.fe_cuda_restore_solution(sys_._h))
    u0 = torch.from_numpy(sys_.getSolution()).pin_memory()
    hostbuf = torch.empty(sys_.nDofs, dtype=torch.float64).pin_memory()
    pu0, pout = C.c_void_p(u0.data_ptr()), C.c_void_p(hostbuf.data_ptr())
    sys_.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        check(lib.fe_cuda_set_solution(sys_._h, pu0, None))
        fe.solveNewtonRaphson(sys_, None, nl)
        check(lib.fe_cuda_get_solution(sys_._h, pout))
    dt = (time.perf_counter() - t0) / steps
    return dt, sys_.nDofs * 8, sys_.nDofs * 8


def algorithmic_bytes(sys_, nvert, precision):
    """Per-launch algorithmic bytes (byte model of the assembly and SpMV roofline):
      assembly  nnz s_A + nElm n_loc 4 + nVert d 8 + nDofs 8 k_in + nInc 8
      SpMV      nnz (s_A + 4) + (nInc + 1) 4 + nInc (s_x + s_y)"""
    sA = 4 if precision == "mixed" else 8
    nl = 15
    res = sys_.nElm * nl * 4 + nvert * 2 * 8 + sys_.nDofs * 8 + sys_.nInc * 8
    mat = sys_.nnz * sA + sys_.nElm * nl * 4 + nvert * 2 * 8 + sys_.nDofs * 8
    sx = 4 if precision == "mixed" else 8   # the Arnoldi SpMV: FP32 vectors (mixed), FP64 (plain)
    spmv = sys_.nnz * (sA + 4) + (sys_.nInc + 1) * 4 + sys_.nInc * 2 * sx
    from feng_gb300._lib import check
    out = {"residual_assembly": res, "matrix_assembly": mat, "spmv": spmv}
    for which, name in ((4, "smoother_step"), (5, "gs_dots"), (6, "gs_update")):
        if which > 4 and precision != "mixed":
            continue
        b = C.c_int64()
        check(sys_.lib.fe_cuda_phase_bytes(sys_._h, which, C.byref(b)))
        out[name] = b.value
    return out


def ncu_traffic(kernel):
    """DRAM bytes per launch of a kernel from the committed ncu summary
    (profiles/ncu_traffic.json), or None."""
    p = ROOT / "profiles" / "ncu_traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text()).get(kernel)
    return None if d is None else d.get("dram_bytes_per_launch")


def phase_bench(sys_, mixed, reps=20):
    """Device-timed phases (L2 flushed before each run): assembly, SpMV, one
    preconditioner application, the finest-level pre-smoothing pass, and for
    the mixed path the two Gram-Schmidt passes at restart/2 = 25 columns
    (the mean column count of a 50-step cycle)."""
    from feng_gb300._lib import check
    out = {}
    phases = [(0, "residual_assembly"), (1, "matrix_assembly"), (2, "spmv"), (3, "preconditioner"),
              (4, "smoother_step")] + ([(5, "gs_dots"), (6, "gs_update")] if mixed else [])
    for which, name in phases:
        ms = C.c_double()
        check(sys_.lib.fe_cuda_bench_phase(sys_._h, which, reps, 256 << 20, C.byref(ms)))
        out[name] = ms.value
    return out


def cpu_baseline(num, forms, gpu_newton_its, gpu_krylov_its, budget_s=20.0):
    """The oracle (C restatement of the reference CPU algorithms, OpenMP) on a
    bounded sample of the workload: full residual + Jacobian assembly of the
    mesh, and FGMRES iterations with block-Jacobi ILU(0) (the reference's
    preconditioner family; it does not converge on this saddle-point system,
    so its per-iteration cost is timed over a fixed count).  Newton-step
    seconds = Newton iterations x assembly + Krylov iterations x per-iteration
    cost, with the GPU run's iteration counts."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import OracleProblem
    from feng_gb300.api import quadrature_rule
    st = num.setup(256)
    arr = num.mesh.arrays()
    tri = arr["tri"]
    xy = np.stack([arr["x"][tri[:, 0]], arr["y"][tri[:, 0]], arr["x"][tri[:, 1]], arr["y"][tri[:, 1]],
                   arr["x"][tri[:, 2]], arr["y"][tri[:, 2]]], 1)
    ia, ja = st.pattern()
    off, el = st.coloring()
    op = OracleProblem(2, st.elementDofs(), xy, st.nInc, st.nDofs, off, el, ia, ja, quadrature_rule(8),
                       [f.sysElm for f in forms])
    u = bc_state(st)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    vals = op.matrix(u, nthreads=cores)
    rhs = op.residual(u, nthreads=cores)
    t_asm = time.perf_counter() - t0
    iters = 20
    t0 = time.perf_counter()
    _, info = op.solve(vals, rhs, method=1, restart=50, max_iter=iters, rtol=1e-30, pc_kind=1,
                       block_of_row=st.blocks(), nthreads=cores)
    t_it = (time.perf_counter() - t0) / max(info["iterations"], 1)
    est = gpu_newton_its * t_asm + gpu_krylov_its * t_it
    return {"value": est, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"oracle port on {cores} threads: one full residual+Jacobian assembly "
                       f"({t_asm:.3f} s, {op.n_elm / t_asm / 1e6:.3f} Melem/s) and {info['iterations']} FGMRES(50)"
                       f"+block-Jacobi-ILU(0) iterations ({t_it * 1e3:.2f} ms each), scaled to the GPU run's "
                       f"{gpu_newton_its} Newton / {gpu_krylov_its} Krylov iterations"),
            "assembly_melem_s": op.n_elm / t_asm / 1e6}


def bc_state(st):
    """Zero unknowns, Kovasznay values on the essential DOFs (nodewise, as
    feSolution::initializeEssentialBC)."""
    from feng_gb300 import exact
    x, y, fld, comp, _ = st.dofInfo()
    u = np.zeros(st.nDofs)
    ess = np.arange(st.nInc, st.nDofs)
    ux, uy = exact.kovasznay_velocity(RE)(x[ess], y[ess])
    (pp,) = exact.kovasznay_pressure(RE)(x[ess], y[ess])
    u[ess] = np.where(fld[ess] == 1, pp, np.where(comp[ess] == 0, ux, uy))
    return u


def reference_arm(args, ws, rank):
    """CPU oracle timed on the host cores, same config and metric."""
    if rank != 0:
        return
    m, num, forms = build_problem(args.n)
    # Iteration counts of the plain method, fixed from the GPU runs of this
    # workload (4 Newton / 1158 Krylov iterations at 256^2), so every step is
    # a bounded CPU sample.
    newton_its, krylov_its = 4, 1158
    vals = []
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(num, forms, newton_its, krylov_its)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = statistics.mean(vals)
    cb["value"] = v
    st = num.setup()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.n, st), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def transient_leg(steps, n=384, re=1000.0, dt=0.005):
    """Config C4: lid-driven cavity from rest, BDF2, 40 steps.  Arms: the
    plain FP64 solver with the reference's guess (previous solution), and the
    mixed solver with the extrapolated and with the learned guess (MLP trained
    online from step 10, used from step 15).  Means over steps 20..steps."""
    from feng_gb300 import cavity
    out = {"workload": f"cavity_re{re:g}_{n}x{n}_dt{dt:g}_bdf2_{steps}steps", "summary_steps": f"20-{steps}"}
    arms = (("plain_fp64_previous", "previous", "fp64", {}),
            ("mixed_extrapolate", "extrapolate", "mixed", {}),
            ("mixed_learned", "learned", "mixed", {"trainFrom": 10, "useFrom": 15}))
    for name, guess, prec, learn in arms:
        _, stats = cavity.run(n, re, dt, steps, guess, prec, **learn)
        out[name] = cavity.summarize(stats, 20)
    p, lrn = out["plain_fp64_previous"].get("step_ms"), out["mixed_learned"].get("step_ms")
    out["speedup_mixed_learned_vs_plain_fp64"] = p / lrn if p and lrn else None
    return out


def workload_config(n, st):
    return {"workload": f"kovasznay_re40_{n}x{n}_p2p1_steady_newton", "cells": n * n,
            "elements": st.nElm, "unknowns": st.nInc, "dofs": st.nDofs, "nnz": st.nnz,
            "quadrature_degree": 8, "stop": "||R||inf/||R0||inf <= 1e-8",
            "inputs_larger_than_l2": True, "parallelism": "replicas"}


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, ws, rank)
        return
    from feng_gb300 import build
    build.build()
    import feng_gb300 as fe  # noqa: F401
    from feng_gb300._lib import check, load
    lib = load()
    check(lib.fe_cuda_set_device(local))
    dist = Dist(ws)
    m, num, forms = build_problem(args.n)
    nvert = m.sizes()[0]

    plain, sol_p = make_system(num, forms, "fp64")
    mixed, sol_m = make_system(num, forms, "mixed")
    clk = Clocks(local)
    t_plain, st_plain, l_plain, ph_plain = timed_steps(plain, newton_opts("fp64"), args.steps, args.warmup, dist)
    t_mixed, st_mixed, l_mixed, ph_mixed = timed_steps(mixed, newton_opts("mixed"), args.steps, args.warmup, dist)
    clocks = clk.stop()
    t_plain = dist.max(t_plain)
    t_mixed = dist.max(t_mixed)
    steps_total = dist.sum(args.steps)
    value = t_mixed / args.steps          # seconds per Newton solve (per replica)
    plain_s = t_plain / args.steps
    e2e_s, h2d, d2h = e2e_steps(mixed, newton_opts("mixed"), max(1, args.steps))
    e2e_s = dist.max(e2e_s)

    # Assembly throughput inside the Newton steps (residual + Jacobian per iteration).
    def asm_rate(st_list, ph, nelm):
        its = sum(s["iterations"] for s in st_list)
        asm_ms = ph["residual_ms"] + ph["matrix_ms"]
        return nelm * its / (asm_ms / 1e3) / 1e6 if asm_ms > 0 else None

    # Per-kernel roofline (device-timed, L2 flushed before each run).
    peak, peak_kind = measured_peaks()
    kern = {}
    for name, sys_, prec in (("fp64", plain, "fp64"), ("mixed", mixed, "mixed")):
        ph = phase_bench(sys_, prec == "mixed")
        by = algorithmic_bytes(sys_, nvert, prec)
        kern[name] = {k: {"ms": ph[k], "bytes": by.get(k),
                          "gbs": (by[k] / (ph[k] / 1e3) / 1e9) if k in by else None} for k in ph}
    # dominant phase of the headline arm inside the Newton step
    ph = ph_mixed
    shares = {"assembly": ph["residual_ms"] + ph["matrix_ms"], "krylov_solve": ph["solve_ms"],
              "preconditioner_build": ph["factor_ms"]}
    # The dominant kernel of the Newton step (the Krylov solve is ~97% of it,
    # and its largest kernel by time is the Gram-Schmidt dot pass): k_gs_dots
    # at the mean column count of a restart cycle.
    def roofline(key, kernel, traffic_key):
        k = kern["mixed"][key]
        return {"kernel": kernel, "bound": "hbm", "achieved": k["gbs"], "peak": peak, "unit": "GB/s",
                "frac": k["gbs"] / peak, "peak_source": peak_kind, "bytes_per_launch": k["bytes"],
                "ms_per_launch": k["ms"], "traffic": ncu_traffic(traffic_key)}
    roof = roofline("gs_dots", "k_gs_dots (FP32 Gram-Schmidt dot pass, 25 basis vectors)", "k_gs_dots@25")
    roof_gsu = roofline("gs_update", "k_gs_upd<32,true> (FP32 Gram-Schmidt update + norm, 25 basis vectors)",
                        "k_gs_upd<32,true>@25")
    roof_sm = roofline("smoother_step", "k_cheb_first_sell<float,2> (finest AMG level, both velocity components)",
                       "k_cheb_first_sell<float,2>")
    asm = kern["mixed"]["matrix_assembly"]
    roof_asm = {"kernel": "k_pack_th + k_matrix_th_rows<float> (row-owned Jacobian assembly)", "bound": "hbm",
                "achieved": asm["gbs"], "peak": peak, "unit": "GB/s", "frac": asm["gbs"] / peak,
                "peak_source": peak_kind, "traffic": ncu_traffic("k_matrix_th_rows<float>")}
    sp = kern["mixed"]["spmv"]
    roof_spmv = {"kernel": "k_spmv_sell (FGMRES inner SpMV, sliced ELL, FP32)", "bound": "hbm", "achieved": sp["gbs"],
                 "peak": peak, "unit": "GB/s", "frac": sp["gbs"] / peak, "peak_source": peak_kind,
                 "traffic": ncu_traffic("k_spmv_sell")}

    nits_p = round(statistics.mean(s["iterations"] for s in st_plain), 2)
    kits_p = round(statistics.mean(s["krylov_iterations"] for s in st_plain), 1)
    nits_m = round(statistics.mean(s["iterations"] for s in st_mixed), 2)
    kits_m = round(statistics.mean(s["krylov_iterations"] for s in st_mixed), 1)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded jittered mesh, Kovasznay BCs)",
        "config": workload_config(args.n, num.setup()),
        "plain_fp64": {"newton_step_s": plain_s, "newton_iterations": nits_p, "krylov_iterations": kits_p,
                       "assembly_melem_s": asm_rate(st_plain, ph_plain, plain.nElm),
                       "final_rel_residual": max(s["residual"] / s["residual0"] for s in st_plain)},
        "mixed": {"newton_step_s": value, "newton_iterations": nits_m, "krylov_iterations": kits_m,
                  "assembly_melem_s": asm_rate(st_mixed, ph_mixed, mixed.nElm),
                  "final_rel_residual": max(s["residual"] / s["residual0"] for s in st_mixed)},
        "speedup_mixed_vs_fp64": plain_s / value,
        "phase_share_ms": shares,
        "kernels": kern,
        "roofline": roof, "roofline_gs_update": roof_gsu, "roofline_smoother": roof_sm,
        "roofline_assembly": roof_asm, "roofline_spmv": roof_spmv,
        "e2e": {"value": e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": l_mixed,
        "gpu_launches_plain_fp64": l_plain,
        "clocks": clocks,
        "units_total": steps_total,
    }
    if args.transient_steps > 0:
        line["transient"] = transient_leg(args.transient_steps)
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(num, forms, nits_p, kits_p)
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()


if __name__ == "__main__":
    main()
