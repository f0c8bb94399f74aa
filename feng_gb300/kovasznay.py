"""Steady Navier-Stokes Kovasznay case through the feNG-style API, and a
command line that runs Newton solves of it on the GPU.

The case: Kovasznay flow at Re on [-0.5, 1.5]^2, an n x n grid with two
triangles per cell, interior vertices jittered by +-0.1 h (SplitMix64, seed
1), Taylor-Hood P2-P1, velocity Dirichlet on "Bord", pressure fixed at
"PointPression", quadrature of degree 8; forms as in the reference's
Navier-Stokes tests (tests/withLinearSolver/navier_stokes.cpp): convective
acceleration (c = -1), mixed divergence (c = 1), divergence of the Newtonian
stress (c = 1, mu = 1/Re).

    python -m feng_gb300.kovasznay --n 256 --precision mixed --solves 1

prints one JSON line with the wall time of each solve and the iteration
counts.  Set FENG_CUDA_GRAPHS=0 to launch the FGMRES restart cycles kernel by
kernel (for per-kernel profiler launch lists).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

DOMAIN = (-0.5, 1.5, -0.5, 1.5)


def build(n: int, re: float = 40.0, jitter: float = 0.1, seed: int = 1):
    """Mesh, numbering and the three bilinear forms of the case."""
    from . import api as fe
    from . import exact
    m = fe.Mesh2DP1.generate_square(n, *DOMAIN, jitter=jitter, seed=seed)
    uex, pex = exact.kovasznay_velocity(re), exact.kovasznay_pressure(re)
    u = fe.createFiniteElementSpace(m, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 8, uex)
    uB = fe.createFiniteElementSpace(m, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 8, uex)
    p = fe.createFiniteElementSpace(m, fe.LAGRANGE, 1, "P", "Domaine", 8, pex)
    pP = fe.createFiniteElementSpace(m, fe.LAGRANGE, 1, "P", "PointPression", 8, pex)
    num = fe.feMetaNumber(m, [u, uB, p, pP], [uB, pP])
    forms = [fe.createBilinearForm([u], fe.feSysElm_VectorConvectiveAcceleration(-1.0)),
             fe.createBilinearForm([p, u], fe.feSysElm_MixedDivergence(1.0)),
             fe.createBilinearForm([u, p], fe.feSysElm_DivergenceNewtonianStress(1.0, 1.0 / re))]
    return m, num, forms


def make_system(num, forms, precision: str, precond: str = "amg", **solver):
    """Linear system (FP64 or mixed) with the boundary values set; extra
    keywords go to LinearSolverOptions (restart, mg_smooth, ...)."""
    from . import api as fe
    opts = fe.LinearSolverOptions(precond=precond, rel_tol=1e-8, max_iter=3000,
                                  precision="mixed" if precision == "mixed" else "fp64", **solver)
    sys_ = fe.createLinearSystem(fe.CUDA, forms, num, opts)
    sol = fe.feSolution(sys_)
    sol.initializeEssentialBC()
    return sys_, sol


def newton_options(precision: str):
    """Stop at ||R||_inf / ||R_0||_inf <= 1e-8; the mixed arm solves inexactly
    (linear tolerance max(1e-6, min(1e-2, 0.1 ||R||/||R_0||)))."""
    from . import api as fe
    if precision == "mixed":
        return fe.feNLSolverOptions(tolResidual=0.0, tolCorrection=0.0, maxIter=30, relResidual=1e-8,
                                    linearRtolMin=1e-6)
    return fe.feNLSolverOptions(tolResidual=0.0, tolCorrection=0.0, maxIter=30, relResidual=1e-8)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=256, help="cells per side")
    ap.add_argument("--re", type=float, default=40.0)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--precond", default="amg", choices=["amg", "ilu0", "bjacobi-ilu0", "jacobi", "none"])
    ap.add_argument("--solves", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=0)
    ap.add_argument("--max-iter", type=int, default=30, help="Newton iterations at most (feNLSolverOptions.maxIter)")
    ap.add_argument("--restart", type=int, default=50, help="FGMRES restart length")
    ap.add_argument("--mg-smooth", type=int, default=1, help="Chebyshev smoother degree of the multigrid")
    ap.add_argument("--gs-passes", type=int, default=1,
                    help="mixed FGMRES Gram-Schmidt: 1 adaptive, 2 always twice, 3 adaptive with the Pythagoras norm")
    ap.add_argument("--phases", default="",
                    help="after the solves, time these benchmark phases (comma list of fe_cuda_bench_phase "
                         "numbers: 0 residual, 1 Jacobian, 2 SpMV, 3 preconditioner, 4 finest smoother pass, "
                         "5 Gram-Schmidt dots, 6 Gram-Schmidt update, 7 and 8 the same two streamed back to back, "
                         "9 the dot pass of 5 by column groups, 11 the preconditioner in a CUDA graph, "
                         "12 one Arnoldi step of a restart cycle replayed from its graph)")
    ap.add_argument("--phase-reps", type=int, default=20)
    ap.add_argument("--errors", action="store_true",
                    help="after the solves, L2 errors of velocity and pressure against the exact Kovasznay flow "
                         "(feNorm VECTOR_L2_ERROR / L2_ERROR on the device)")
    ap.add_argument("--vtk", default="",
                    help="after the solves, write the solution to this legacy VTK file (feExporterVTK layout)")
    args = ap.parse_args(argv)

    from . import api as fe
    from ._lib import check
    ts0 = time.perf_counter()
    mesh, num, forms = build(args.n, args.re)
    ts1 = time.perf_counter()
    check(fe._lib.load().fe_cuda_set_device(0))  # CUDA context creation, timed apart
    ts2 = time.perf_counter()
    sys_, _ = make_system(num, forms, args.precision, args.precond, restart=args.restart,
                          mg_smooth=args.mg_smooth, gs_passes=args.gs_passes)
    sys_.synchronize()
    ts3 = time.perf_counter()
    nl = newton_options(args.precision)
    nl.maxIter = args.max_iter
    lib = sys_.lib
    check(lib.fe_cuda_save_solution(sys_._h))
    runs = []
    for i in range(args.warmup + args.solves):
        check(lib.fe_cuda_restore_solution(sys_._h))
        sys_.synchronize()
        t0 = time.perf_counter()
        st = fe.solveNewtonRaphson(sys_, None, nl)
        sys_.synchronize()
        if i >= args.warmup:
            runs.append({"seconds": time.perf_counter() - t0, "newton_iterations": st["iterations"],
                         "krylov_iterations": st["krylov_iterations"],
                         "rel_residual": st["residual"] / st["residual0"] if st["residual0"] else 0.0})
    errors = {}
    if args.errors and runs:
        from . import exact
        sol = fe.feSolution(sys_)
        sol.pull()
        uS = next(sp for f in forms for sp in f.spaces if sp.element == fe.VECTOR_LAGRANGE)
        pS = next(sp for f in forms for sp in f.spaces if sp.element == fe.LAGRANGE)
        errors = {"u_l2": fe.createNorm(fe.VECTOR_L2_ERROR, [uS], sol, None, exact.kovasznay_velocity(args.re)).compute(),
                  "p_l2": fe.createNorm(fe.L2_ERROR, [pS], sol, exact.kovasznay_pressure(args.re)).compute()}
    if args.vtk and runs:
        fe.createVisualizationExporter(fe.VTK, num, sys_.getSolution(), mesh, num.spaces).writeStep(args.vtk)
    phases = {}
    for w in [int(v) for v in args.phases.split(",") if v.strip()]:
        # device time per run with the L2 flushed before each run; bytes:
        # algorithmic bytes where the library defines them (phases 4-8)
        ms = C.c_double()
        check(lib.fe_cuda_bench_phase(sys_._h, w, args.phase_reps, 256 << 20, C.byref(ms)))
        ph = {"us": ms.value * 1e3}
        if 4 <= w <= 9:
            by = C.c_int64()
            check(lib.fe_cuda_phase_bytes(sys_._h, w, C.byref(by)))
            ph["bytes"] = by.value
            ph["gbs"] = by.value / (ms.value * 1e-3) / 1e9
        phases[str(w)] = ph
    print(json.dumps({"case": f"kovasznay_re{args.re:g}_{args.n}x{args.n}", "precision": args.precision,
                      "precond": args.precond, "restart": args.restart, "mg_smooth": args.mg_smooth, "gs_passes": args.gs_passes,
                      "unknowns": sys_.nInc, "nnz": sys_.nnz,
                      "setup_s": {"mesh_numbering_pattern": ts1 - ts0, "cuda_context": ts2 - ts1,
                                  "system_create": ts3 - ts2},
                      "solves": runs, "errors": errors, "phases": phases}))


if __name__ == "__main__":
    main()
