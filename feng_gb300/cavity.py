"""Transient lid-driven cavity through the feNG-style API, and a command line
that runs BDF2 time steps of it on the GPU with the extrapolated or the
learned Newton initial guess.

The case: unit square, an n x n grid with two triangles per cell, interior
vertices jittered by +-0.1 h (SplitMix64), Taylor-Hood P2-P1, lid u = (1, 0)
on y = 1 and no-slip on the other walls (velocity Dirichlet on "Bord"),
pressure fixed at "PointPression", quadrature of degree 8, forms and signs of
the reference's unsteady Navier-Stokes test
(tests/withLinearSolver/vectorFEunsteady.cpp:560-584): transient mass (1),
convective acceleration (1), divergence of the Newtonian stress (-1, mu =
1/Re), mixed divergence (1).  Starts from rest.

    python -m feng_gb300.cavity --n 384 --re 1000 --dt 0.005 --steps 40 --guess learned

prints one JSON line with per-step statistics and their summary.
"""
from __future__ import annotations

import argparse
import json
import statistics


def build(n: int, re: float, jitter: float = 0.1, seed: int = 1):
    """Mesh, numbering and the four bilinear forms of the cavity."""
    from . import api as fe
    from . import exact
    m = fe.Mesh2DP1.generate_square(n, 0.0, 1.0, 0.0, 1.0, jitter=jitter, seed=seed)
    lid = exact.cavity_lid()
    u = fe.createFiniteElementSpace(m, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 8, lid)
    uB = fe.createFiniteElementSpace(m, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 8, lid)
    p = fe.createFiniteElementSpace(m, fe.LAGRANGE, 1, "P", "Domaine", 8, exact.zero_scalar)
    pP = fe.createFiniteElementSpace(m, fe.LAGRANGE, 1, "P", "PointPression", 8, exact.zero_scalar)
    num = fe.feMetaNumber(m, [u, uB, p, pP], [uB, pP])
    forms = [fe.createBilinearForm([u], fe.feSysElm_TransientVectorMass(1.0)),
             fe.createBilinearForm([u], fe.feSysElm_VectorConvectiveAcceleration(1.0)),
             fe.createBilinearForm([p, u], fe.feSysElm_MixedDivergence(1.0)),
             fe.createBilinearForm([u, p], fe.feSysElm_DivergenceNewtonianStress(-1.0, 1.0 / re))]
    return m, num, forms


def run(n: int, re: float, dt: float, steps: int, guess: str, precision: str = "mixed", solver=None, **learn):
    """BDF2 steps from rest; returns (system, per-step statistics).  solver:
    extra LinearSolverOptions keywords."""
    from . import api as fe
    _, num, forms = build(n, re)
    opts = fe.LinearSolverOptions(precond="amg", rel_tol=1e-8, max_iter=3000,
                                  precision="mixed" if precision == "mixed" else "fp64", **(solver or {}))
    sys_ = fe.createLinearSystem(fe.CUDA, forms, num, opts)
    sol = fe.feSolution(sys_)
    sol.initializeEssentialBC()
    nl = fe.feNLSolverOptions(tolResidual=0.0, tolCorrection=0.0, tolDivergence=1e12, maxIter=30,
                              relResidual=1e-8, linearRtolMin=1e-6 if precision == "mixed" else 0.0)
    ti = fe.createTimeIntegrator(fe.BDF2, nl, sys_, sol, 0.0, steps * dt, steps, guess=guess, **learn)
    return sys_, ti.makeSteps(steps)


def summarize(stats, first: int):
    """Means over the converged steps >= first (1-based); steps whose status
    is not 0 are counted in failed_steps and left out of the means."""
    failed = sum(1 for s in stats if s["step"] >= first and s["status"] != 0)
    late = [s for s in stats if s["step"] >= first and s["status"] == 0]
    if not late:
        return {"steps": 0, "failed_steps": failed}
    return {"steps": len(late), "failed_steps": failed,
            "step_ms": statistics.mean(s["step_ms"] for s in late),
            "newton_iterations": statistics.mean(s["newton_iterations"] for s in late),
            "krylov_iterations": statistics.mean(s["krylov_iterations"] for s in late),
            "guess_residual_ratio": statistics.mean(s["residual_guess"] / s["residual_ref"] for s in late
                                                    if s["residual_ref"] > 0),
            "learned_used": sum(s["guess_used"] == 2 for s in late),
            "extrap_residual_ratio": statistics.mean(s["residual_extrap"] / s["residual_ref"] for s in late
                                                     if s["residual_ref"] > 0 and s["residual_extrap"] > 0)
            if any(s["residual_extrap"] > 0 for s in late) else None,
            "train_loss": late[-1]["train_loss"],
            "train_ms": statistics.mean(s["train_ms"] for s in late)}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=384)
    ap.add_argument("--re", type=float, default=1000.0)
    ap.add_argument("--dt", type=float, default=0.005)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--guess", default="learned", choices=["previous", "extrapolate", "learned"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--train-from", type=int, default=10)
    ap.add_argument("--use-from", type=int, default=15)
    ap.add_argument("--summary-from", type=int, default=20)
    ap.add_argument("--gs-passes", type=int, default=1,
                    help="mixed FGMRES Gram-Schmidt: 1 adaptive, 2 always twice, 3 adaptive with the Pythagoras norm")
    ap.add_argument("--restart", type=int, default=50)
    ap.add_argument("--train-iters", type=int, default=8, help="Adam steps per time step")
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--batch", type=int, default=16384)
    args = ap.parse_args(argv)
    learn = dict(trainFrom=args.train_from, useFrom=args.use_from, trainIters=args.train_iters, lr=args.lr,
                 batch=args.batch) if args.guess == "learned" else {}
    sys_, stats = run(args.n, args.re, args.dt, args.steps, args.guess, args.precision,
                      solver=dict(gs_passes=args.gs_passes, restart=args.restart), **learn)
    print(json.dumps({"case": f"cavity_re{args.re:g}_{args.n}x{args.n}_dt{args.dt:g}", "guess": args.guess,
                      "precision": args.precision, "summary": summarize(stats, args.summary_from),
                      "phase_ms_total": sys_.times(), "steps": stats}))


if __name__ == "__main__":
    main()
