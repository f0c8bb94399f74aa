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
    ap.add_argument("--transient-steps", type=int, default=400,
                    help="BDF2 steps of the lid-driven cavity leg (configuration C4; 0: skip)")
    ap.add_argument("--c5-steps", type=int, default=50, help="BDF2 steps of the 64^3 tetrahedra leg (mixed arm)")
    ap.add_argument("--legs", type=int, default=1,
                    help="1: also time the diffusion 64x64 (C1), Kovasznay 512x512 (C3) and 64^3 tetrahedra (C5) "
                         "configurations")
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
    for which, name in ((4, "smoother_step"), (5, "gs_dots"), (6, "gs_update"), (7, "gs_dots_stream"),
                        (8, "gs_update_stream"), (9, "gs_dots_groups")):
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
    (the mean column count of a 50-step cycle), each once alone (flushed,
    one launch between two events: the launch latency and the tail are in
    it) and once streamed (10 x reps launches back to back between two
    events over basis copies larger than three L2s: the mean time of a pass
    as it runs inside the Arnoldi loop); the dot pass also by the
    column-group kernel.  In-graph timings: the preconditioner application
    replayed back to back from a CUDA graph, and one Arnoldi step of a full
    FGMRES(50) restart cycle replayed from its graph (all 50 steps run)."""
    from feng_gb300._lib import check
    out = {}
    phases = [(0, "residual_assembly"), (1, "matrix_assembly"), (2, "spmv"), (3, "preconditioner"),
              (4, "smoother_step"), (11, "preconditioner_in_graph"), (12, "arnoldi_step_in_graph")] + (
                  [(5, "gs_dots"), (6, "gs_update"), (7, "gs_dots_stream"), (8, "gs_update_stream"),
                   (9, "gs_dots_groups")] if mixed else [])
    for which, name in phases:
        ms = C.c_double()
        check(sys_.lib.fe_cuda_bench_phase(sys_._h, which, reps, 256 << 20, C.byref(ms)))
        out[name] = ms.value
    return out


def oracle_problem(n):
    """The C2 problem built by the oracle alone (its own set-up, element
    kernels and solver; nothing of the product is loaded)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from newton_oracle import Problem2D
    return Problem2D("ns_kovasznay", n, RE)


def oracle_solve(pb, nthreads):
    from newton_oracle import newton_solve
    return newton_solve(pb, rel=1e-8, linear_rtol=1e-8, restart=50, nthreads=nthreads)


def cpu_baseline(n):
    """One complete CPU Newton solve of the workload by the oracle (its own
    set-up; FP64 assembly with the reference's element kernels and colored
    scatter; FGMRES(50) with the saddle-point multigrid preconditioner at the
    reference's linear tolerance 1e-8; stop ||R||inf <= 1e-8 ||R0||inf) on
    all host threads, timed end to end (set-up excluded)."""
    cores = os.cpu_count() or 1
    pb = oracle_problem(n)
    u, st = oracle_solve(pb, cores)
    melem = pb.n_elm * st["newton_iterations"] / max(st["residual_s"] + st["matrix_s"], 1e-12) / 1e6
    return {"value": st["seconds"], "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"one complete Newton solve of the workload by the oracle port on {cores} threads: "
                       f"{st['newton_iterations']} Newton / {st['krylov_iterations']} FGMRES(50) iterations "
                       f"(saddle-point multigrid preconditioner, FP64), final relative residual "
                       f"{st['final_rel_residual']:.2e}"),
            "newton_iterations": st["newton_iterations"], "krylov_iterations": st["krylov_iterations"],
            "phase_s": {k: st[k] for k in ("residual_s", "matrix_s", "factor_s", "solve_s")},
            "assembly_melem_s": melem}, u


def reference_arm(args, ws, rank):
    """The reference's CPU path as the oracle restates it, timed on the host
    cores: every step is one complete Newton solve of the workload (no
    iteration count borrowed, nothing scaled).  Only rank 0 works."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    pb = oracle_problem(args.n)
    times, stats = [], []
    for i in range(args.warmup + args.steps):
        _, st = oracle_solve(pb, cores)
        if not st["converged"]:
            raise RuntimeError(f"oracle Newton solve did not converge: {st}")
        if i >= args.warmup:
            times.append(st["seconds"])
            stats.append(st)
    v = statistics.mean(times)
    # A one-thread sample: one residual + Jacobian assembly and one FGMRES
    # restart cycle (50 iterations) of the first Newton step.
    from newton_oracle import one_thread_sample
    one = one_thread_sample(pb)
    cb = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
          "sample": (f"each step one complete Newton solve by the oracle port on {cores} threads: "
                     f"{stats[0]['newton_iterations']} Newton / {stats[0]['krylov_iterations']} FGMRES(50) "
                     f"iterations, saddle-point multigrid preconditioner, FP64"),
          "one_thread": one}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.n, pb.n_elm, pb.n_inc, pb.n_dofs, pb.nnz),
            "newton_iterations": statistics.mean(s["newton_iterations"] for s in stats),
            "krylov_iterations": statistics.mean(s["krylov_iterations"] for s in stats),
            "final_rel_residual": max(s["final_rel_residual"] for s in stats),
            "phase_s": {k: statistics.mean(s[k] for s in stats) for k in ("residual_s", "matrix_s", "factor_s",
                                                                          "solve_s")},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def c1_leg(n=64, reps=5):
    """Config C1: steady P2 diffusion on the 64 x 64 mesh, FP64, Newton (one
    linear solve) to ||R||inf <= 1e-10 ||R0||inf with CG at rel 1e-10:
    ILU(0) (the configuration's preconditioner) and the multigrid.  Error of
    the solution against the oracle's CPU solve of the same system."""
    import feng_gb300 as fe
    from feng_gb300 import exact
    sys.path.insert(0, str(ROOT / "oracle"))
    from newton_oracle import Problem2D, newton_solve
    out = {"workload": f"diffusion_p2_{n}x{n}_cg_rel1e-10"}
    pb = Problem2D("diffusion", n)
    u_or, st_or = newton_solve(pb, rel=1e-10, linear_rtol=1e-10, precond="ilu0")
    out["oracle_cpu_cg_ilu0"] = {"seconds": st_or["seconds"], "krylov_iterations": st_or["krylov_iterations"],
                                 "threads": st_or["threads"]}
    m = fe.Mesh2DP1.generate_square(n, 0.0, 1.0, 0.0, 1.0, jitter=0.1, seed=1)
    u = fe.createFiniteElementSpace(m, fe.LAGRANGE, 2, "U", "Domaine", 4, exact.zero_scalar)
    uB = fe.createFiniteElementSpace(m, fe.LAGRANGE, 2, "U", "Bord", 4, exact.sin_sin)
    num = fe.feMetaNumber(m, [uB, u], [uB])
    forms = [fe.createBilinearForm([u], fe.feSysElm_Diffusion(1.0)),
             fe.createBilinearForm([u], fe.feSysElm_Source(fe.api.SRC_SIN_SIN, (-2 * np.pi ** 2,)))]
    nl = fe.feNLSolverOptions(tolResidual=0.0, tolCorrection=0.0, maxIter=10, relResidual=1e-10)
    for pc in ("ilu0", "amg"):
        sys_ = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(krylov="cg", precond=pc,
                                                                              rel_tol=1e-10, max_iter=5000))
        sol = fe.feSolution(sys_)
        sol.initializeEssentialBC()
        secs, its = [], []
        for i in range(reps + 1):
            sol.initializeEssentialBC()
            sol.u[:sys_.nInc] = 0.0
            sol.push()
            sys_.synchronize()
            t0 = time.perf_counter()
            st = fe.solveNewtonRaphson(sys_, None, nl)
            sys_.synchronize()
            if i > 0:
                secs.append(time.perf_counter() - t0)
                its.append(st["krylov_iterations"])
            if st["return"] != 0:
                raise RuntimeError(f"C1 solve failed ({pc}): {st}")
        ug = sys_.getSolution()
        out[f"gpu_cg_{pc}"] = {"newton_step_s": statistics.mean(secs), "krylov_iterations": statistics.mean(its),
                               "error_vs_oracle": float(np.max(np.abs(ug - u_or)) / np.max(np.abs(u_or)))}
    return out


def c3_leg(n=512, reps=2):
    """Config C3: Kovasznay on the 512 x 512 mesh, mixed and plain FP64
    Newton solves to ||R||inf <= 1e-8 ||R0||inf; iteration counts, L2 errors
    against the exact flow (device feNorm) and the difference of the mixed
    solution from the FP64 one."""
    import feng_gb300 as fe
    from feng_gb300 import exact, kovasznay
    m, num, forms = kovasznay.build(n, RE)
    out = {"workload": f"kovasznay_re40_{n}x{n}_p2p1_steady_newton", "elements": 2 * n * n}
    sols = {}
    for prec in ("mixed", "fp64"):
        sys_, sol = kovasznay.make_system(num, forms, prec)
        lib = sys_.lib
        from feng_gb300._lib import check
        check(lib.fe_cuda_save_solution(sys_._h))
        secs = []
        for i in range(reps + 1):
            check(lib.fe_cuda_restore_solution(sys_._h))
            sys_.synchronize()
            t0 = time.perf_counter()
            st = fe.solveNewtonRaphson(sys_, None, kovasznay.newton_options(prec))
            sys_.synchronize()
            if st["return"] != 0:
                raise RuntimeError(f"C3 solve failed ({prec}): {st}")
            if i > 0:
                secs.append(time.perf_counter() - t0)
        sol.pull()
        uS = next(sp for f in forms for sp in f.spaces if sp.element == fe.VECTOR_LAGRANGE)
        pS = next(sp for f in forms for sp in f.spaces if sp.element == fe.LAGRANGE)
        sols[prec] = sys_.getSolution()
        out[prec] = {"newton_step_s": statistics.mean(secs), "newton_iterations": st["iterations"],
                     "krylov_iterations": st["krylov_iterations"],
                     "final_rel_residual": st["residual"] / st["residual0"],
                     "l2_error_u": fe.createNorm(fe.VECTOR_L2_ERROR, [uS], sol, None,
                                                 exact.kovasznay_velocity(RE)).compute(),
                     "l2_error_p": fe.createNorm(fe.L2_ERROR, [pS], sol, exact.kovasznay_pressure(RE)).compute()}
        del sys_, sol
    out["mixed_vs_fp64_rel_diff"] = float(np.max(np.abs(sols["mixed"] - sols["fp64"])) / np.max(np.abs(sols["fp64"])))
    out["speedup_mixed_vs_fp64"] = out["fp64"]["newton_step_s"] / out["mixed"]["newton_step_s"]
    return out


def c5_leg(n=64, reps=5, steps=50, steps_fp64=10):
    """Config C5's system on the device: the unit cube, n^3 cells of 6 Kuhn
    tetrahedra jittered by +-0.05 h (seed 1), P2-P1 Taylor-Hood with the
    unsteady Navier-Stokes forms (transient mass, convection at Re 100,
    stress, divergence, body force sin(pi x) sin(pi y) sin(pi z) in x),
    degree-5 rule (exact for the forms' polynomial integrands).  Times the
    host set-up, the system creation (device element-to-nonzero map), and
    residual and Jacobian assembly (FP64 and mixed: FP32 Jacobian) with the
    L2 flushed before each run.  Assembly bytes per launch:
    nnz s_A + nElm 34 4 + nVert 3 8 + nDofs 8 k_in + nInc 8."""
    import feng_gb300 as fe
    from feng_gb300._lib import check
    out = {"workload": f"cube_{n}^3_kuhn_tets_p2p1_navier_stokes_re100_dt0.01"}
    from feng_gb300 import cube
    t0 = time.perf_counter()
    mesh, num, forms = cube.build(n, 100.0)
    out["host_setup_s"] = time.perf_counter() - t0
    out["pattern_on_device"] = num.setup().patternOnDevice
    nvert = mesh.sizes()[0]
    peak, peak_kind = measured_peaks()
    for prec in ("fp64", "mixed"):
        t0 = time.perf_counter()
        sys_ = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond="jacobi", precision=prec))
        sys_.synchronize()
        create_s = time.perf_counter() - t0
        rng = np.random.default_rng(1)
        sys_.setSolution(rng.uniform(-1, 1, sys_.nDofs), rng.uniform(-1, 1, sys_.nDofs))
        sys_.setTime(0.0, 300.0)
        ph = {}
        for which, name in ((0, "residual"), (1, "jacobian")):
            ms = C.c_double()
            check(sys_.lib.fe_cuda_bench_phase(sys_._h, which, reps, 256 << 20, C.byref(ms)))
            ph[name] = ms.value
        sA = 8 if prec == "fp64" else 4
        base = sys_.nElm * 34 * 4 + nvert * 3 * 8 + sys_.nDofs * 8 * 2
        by = {"residual": base + sys_.nInc * 8, "jacobian": sys_.nnz * sA + base}
        route = sys_.jacobianRoute
        out[prec] = {"system_create_s": create_s, "jacobian_route": "row-owned" if route else "colored scatter",
                     "jacobian_kernel": ("k_pack_tet + k_matrix_tet_rows (FP32, warp per velocity node / pressure row)"
                                         if route else f"k_matrix_tet<{'double' if prec == 'fp64' else 'float'}> "
                                         "(colored, L2 reductions through the element-to-nonzero map)"),
                     **{f"{k}_ms": v for k, v in ph.items()},
                     "assembly_melem_s": sys_.nElm / ((ph["residual"] + ph["jacobian"]) / 1e3) / 1e6,
                     "roofline_jacobian": {"bound": "hbm", "bytes_per_launch": by["jacobian"],
                                           "achieved": by["jacobian"] / (ph["jacobian"] / 1e3) / 1e9,
                                           "peak": peak, "unit": "GB/s", "peak_source": peak_kind,
                                           "frac": by["jacobian"] / (ph["jacobian"] / 1e3) / 1e9 / peak}}
        out.update(elements=sys_.nElm, unknowns=sys_.nInc, dofs=sys_.nDofs, nnz=sys_.nnz, colors=sys_.nColors)
        del sys_
    # BDF2 time steps from rest (dt 0.01): mixed with the extrapolated guess,
    # plain FP64 with the reference's (previous solution); Newton to
    # ||R||inf <= 1e-8 ||R(u^n)||inf; the saddle-point multigrid on the three
    # velocity components.  The learned guess is built for triangles.
    from feng_gb300 import cavity, cube
    for prec, guess, nsteps in (("mixed", "extrapolate", steps), ("fp64", "previous", min(steps, steps_fp64))):
        if nsteps <= 0:
            continue
        try:
            t0 = time.perf_counter()
            sys_, stats = cube.run_on(num, forms, 0.01, nsteps, guess, prec, rel=1e-8)
            wall = time.perf_counter() - t0
            summ = cavity.summarize(stats, 3)
            summ.update(steps_run=nsteps, wall_s_with_setup=wall, step_ms_total=sum(x["step_ms"] for x in stats),
                        newton_iterations_total=sum(x["newton_iterations"] for x in stats),
                        krylov_iterations_total=sum(x["krylov_iterations"] for x in stats),
                        # device time of the phases over all steps (CUDA events around each call)
                        phase_ms_total=sys_.times())
            out[f"bdf2_{prec}"] = summ
            del sys_
        except Exception as e:  # recorded, so that the rest of the benchmark line still prints
            out[f"bdf2_{prec}"] = {"error": f"{type(e).__name__}: {e}"}
    return out


def transient_leg(steps, n=384, re=1000.0, dt=0.005):
    """Config C4: lid-driven cavity from rest, BDF2 dt 0.005, `steps` steps.
    Arms: the plain FP64 solver with the reference's guess (previous
    solution), and the mixed solver with the extrapolated and with the
    learned guess (MLP trained online from step 20, used from step 25).
    Means over the converged steps 25..steps; failed steps are counted."""
    from feng_gb300 import cavity
    first = 25
    out = {"workload": f"cavity_re{re:g}_{n}x{n}_dt{dt:g}_bdf2_{steps}steps", "summary_steps": f"{first}-{steps}"}
    arms = (("plain_fp64_previous", "previous", "fp64", {}),
            ("mixed_extrapolate", "extrapolate", "mixed", {}),
            ("mixed_learned", "learned", "mixed", {"trainFrom": 20, "useFrom": 25}))
    for name, guess, prec, learn in arms:
        _, stats = cavity.run(n, re, dt, steps, guess, prec, **learn)
        out[name] = cavity.summarize(stats, first)
        out[name]["newton_iterations_total"] = sum(x["newton_iterations"] for x in stats)
        out[name]["krylov_iterations_total"] = sum(x["krylov_iterations"] for x in stats)
        out[name]["step_ms_total"] = sum(x["step_ms"] for x in stats)
    p, lrn = out["plain_fp64_previous"].get("step_ms"), out["mixed_learned"].get("step_ms")
    out["speedup_mixed_learned_vs_plain_fp64"] = p / lrn if p and lrn else None
    return out


def workload_config(n, n_elm, n_inc, n_dofs, nnz):
    return {"workload": f"kovasznay_re40_{n}x{n}_p2p1_steady_newton", "cells": n * n,
            "elements": n_elm, "unknowns": n_inc, "dofs": n_dofs, "nnz": nnz,
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
    # Plain FP64 with the mixed arm's inexact-Newton forcing: separates what
    # the precision gains from what the forcing gains.
    nl_f = newton_opts("fp64")
    nl_f.linearRtolMin = 1e-6
    t_forc, st_forc, _, _ = timed_steps(plain, nl_f, args.steps, min(args.warmup, 1), dist)
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
    # The dominant kernel of the Newton step: the Krylov solve is ~97% of
    # it, and its largest kernel by device time is the Arnoldi SpMV
    # (k_spmv_sell, one launch per FGMRES iteration; profiles/ holds the
    # launch list with the shares).
    def roofline(key, kernel, traffic_key):
        # the streamed timing (launches back to back over cold data) where the
        # phase has one, with the single flushed launch beside it
        k = kern["mixed"][key]
        ks = kern["mixed"].get(key + "_stream")
        main = ks or k
        out = {"kernel": kernel, "bound": "hbm", "achieved": main["gbs"], "peak": peak, "unit": "GB/s",
               "frac": main["gbs"] / peak, "peak_source": peak_kind, "bytes_per_launch": main["bytes"],
               "ms_per_launch": main["ms"], "traffic": ncu_traffic(traffic_key),
               "timing": "back-to-back launches, working set > 3 x L2" if ks else "one launch, L2 flushed"}
        if ks:
            out["single_launch"] = {"ms": k["ms"], "achieved": k["gbs"], "frac": k["gbs"] / peak}
        return out
    roof = roofline("spmv", "k_spmv_sell (FGMRES inner SpMV, sliced ELL, FP32)", "k_spmv_sell")
    roof_gsd = roofline("gs_dots", "k_gs_dots_all<16> (FP32 Gram-Schmidt dot pass, one pass over w and every "
                        "column, 25 basis vectors)", "k_gs_dots_all@25")
    roof_gsu = roofline("gs_update", "k_gs_upd<32,true> (FP32 Gram-Schmidt update + norm, 25 basis vectors)",
                        "k_gs_upd<32,true>@25")
    roof_sm = roofline("smoother_step", "k_cheb_first_sell<float,2> (finest AMG level, both velocity components)",
                       "k_cheb_first_sell<float,2>")
    asm = kern["mixed"]["matrix_assembly"]
    roof_asm = {"kernel": "k_pack_th + k_matrix_th_rows<float> (row-owned Jacobian assembly)", "bound": "hbm",
                "achieved": asm["gbs"], "peak": peak, "unit": "GB/s", "frac": asm["gbs"] / peak,
                "peak_source": peak_kind, "traffic": ncu_traffic("k_matrix_th_rows<float>")}

    nits_p = round(statistics.mean(s["iterations"] for s in st_plain), 2)
    kits_p = round(statistics.mean(s["krylov_iterations"] for s in st_plain), 1)
    nits_m = round(statistics.mean(s["iterations"] for s in st_mixed), 2)
    kits_m = round(statistics.mean(s["krylov_iterations"] for s in st_mixed), 1)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded jittered mesh, Kovasznay BCs)",
        "config": workload_config(args.n, mixed.nElm, mixed.nInc, mixed.nDofs, mixed.nnz),
        "plain_fp64": {"newton_step_s": plain_s, "newton_iterations": nits_p, "krylov_iterations": kits_p,
                       "assembly_melem_s": asm_rate(st_plain, ph_plain, plain.nElm),
                       "final_rel_residual": max(s["residual"] / s["residual0"] for s in st_plain)},
        "mixed": {"newton_step_s": value, "newton_iterations": nits_m, "krylov_iterations": kits_m,
                  "assembly_melem_s": asm_rate(st_mixed, ph_mixed, mixed.nElm),
                  "final_rel_residual": max(s["residual"] / s["residual0"] for s in st_mixed)},
        "plain_fp64_inexact_newton": {
            "newton_step_s": t_forc / args.steps,
            "newton_iterations": round(statistics.mean(s["iterations"] for s in st_forc), 2),
            "krylov_iterations": round(statistics.mean(s["krylov_iterations"] for s in st_forc), 1),
            "converged": all(s["return"] == 0 for s in st_forc),
            "final_rel_residual": max(s["residual"] / s["residual0"] for s in st_forc),
            "note": "FP64 everywhere, linear tolerance max(1e-6, min(1e-2, 0.1 ||R||/||R0||)) as the mixed arm"},
        "speedup_mixed_vs_fp64": plain_s / value,
        # the mixed arm's speed-up over the plain arm as (cost of one FGMRES
        # iteration, FP64 / mixed) x (FGMRES iterations per solve, plain /
        # mixed: the forcing terms), both from the converged solves above
        "speedup_split": {"precision_per_fgmres_iteration": (plain_s / kits_p) / (value / kits_m),
                          "fgmres_iteration_count_ratio": kits_p / kits_m,
                          "product": (plain_s / kits_p) / (value / kits_m) * (kits_p / kits_m),
                          "note": "plain_fp64_inexact_newton (FP64 with the mixed arm's forcing) is reported "
                                  "but not used here: it does not reach the stop"},
        "phase_share_ms": shares,
        "kernels": kern,
        "roofline": roof, "roofline_gs_dots": roof_gsd, "roofline_gs_update": roof_gsu,
        "roofline_smoother": roof_sm, "roofline_assembly": roof_asm,
        "e2e": {"value": e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": l_mixed,
        "gpu_launches_plain_fp64": l_plain,
        "clocks": clocks,
        "units_total": steps_total,
    }
    u_mixed = mixed.getSolution()
    u_plain = plain.getSolution()
    if args.legs:
        line["c1"] = c1_leg()
        line["c3"] = c3_leg()
        line["c5"] = c5_leg(steps=args.c5_steps)
    if args.transient_steps > 0:
        line["transient"] = transient_leg(args.transient_steps)
    if rank == 0:
        cb, u_oracle = cpu_baseline(args.n)
        line["cpu_baseline"] = cb
        scale = float(np.max(np.abs(u_oracle)))
        line["error_vs_fp64_oracle"] = {
            "mixed": float(np.max(np.abs(u_mixed - u_oracle)) / scale),
            "plain_fp64": float(np.max(np.abs(u_plain - u_oracle)) / scale),
            "definition": "max |u - u_oracle| / max |u_oracle| over all DOFs; both solves stop at "
                          "||R||inf <= 1e-8 ||R0||inf, so this is the algebraic error left at the stop"}
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()


if __name__ == "__main__":
    main()
