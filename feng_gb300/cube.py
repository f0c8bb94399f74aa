"""Unsteady Navier-Stokes in the unit cube on P2-P1 tetrahedra through the
feNG-style API, and a command line that runs BDF2 time steps of it on the GPU.

The case: n^3 cells of 6 Kuhn tetrahedra, interior vertices jittered by
+-0.05 h (SplitMix64), Taylor-Hood P2-P1 with no-slip on every wall
(velocity Dirichlet on "Bord"), the pressure determined up to a constant,
forms with the sign convention of the reference's unsteady Navier-Stokes
test (tests/withLinearSolver/vectorFEunsteady.cpp:560-584): transient mass
(1), convective acceleration (1), divergence of the Newtonian stress (-1,
mu = 1/Re), mixed divergence (1), and the body force
g = (sin(pi x) sin(pi y) sin(pi z), 0, 0) (VectorSource with f = -g, since
the forms carry the force on the residual's side).  Quadrature of degree 5
(exact for every polynomial integrand on affine tetrahedra).  Starts from
rest.

    python -m feng_gb300.cube --n 64 --re 100 --dt 0.01 --steps 50 --precision mixed

prints one JSON line with per-step statistics and their summary.
"""
from __future__ import annotations

import argparse
import json


def build(n: int, re: float, jitter: float = 0.05, seed: int = 1):
    """Mesh, numbering and the five bilinear forms of the case."""
    from . import api as fe
    m = fe.Mesh3DP1.generate_cube(n, jitter=jitter, seed=seed)
    u = fe.createFiniteElementSpace(m, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 5)
    uB = fe.createFiniteElementSpace(m, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 5)
    p = fe.createFiniteElementSpace(m, fe.LAGRANGE, 1, "P", "Domaine", 5)
    num = fe.feMetaNumber(m, [u, uB, p], [uB])
    forms = [fe.createBilinearForm([u], fe.feSysElm_TransientVectorMass(1.0)),
             fe.createBilinearForm([u], fe.feSysElm_VectorConvectiveAcceleration(1.0)),
             fe.createBilinearForm([p, u], fe.feSysElm_MixedDivergence(1.0)),
             fe.createBilinearForm([u, p], fe.feSysElm_DivergenceNewtonianStress(-1.0, 1.0 / re)),
             fe.createBilinearForm([u], fe.feSysElm_VectorSource(fe.SRC_SIN3_BODY, (-1.0,)))]
    return m, num, forms


def make_system(num, forms, precision: str, precond: str = "amg", **solver):
    from . import api as fe
    opts = fe.LinearSolverOptions(precond=precond, rel_tol=1e-8, max_iter=3000,
                                  precision="mixed" if precision == "mixed" else "fp64", **solver)
    sys_ = fe.createLinearSystem(fe.CUDA, forms, num, opts)
    sol = fe.feSolution(sys_)
    sol.initializeEssentialBC()
    return sys_, sol


def run(n: int, re: float, dt: float, steps: int, guess: str, precision: str = "mixed", rel: float = 1e-8,
        solver=None):
    """BDF2 steps from rest; returns (system, per-step statistics)."""
    _, num, forms = build(n, re)
    return run_on(num, forms, dt, steps, guess, precision, rel, solver)


def run_on(num, forms, dt: float, steps: int, guess: str, precision: str = "mixed", rel: float = 1e-8, solver=None):
    """BDF2 steps from rest on a numbering and forms of build()."""
    from . import api as fe
    sys_, sol = make_system(num, forms, precision, **(solver or {}))
    nl = fe.feNLSolverOptions(tolResidual=0.0, tolCorrection=0.0, tolDivergence=1e12, maxIter=30,
                              relResidual=rel, linearRtolMin=1e-6 if precision == "mixed" else 0.0)
    ti = fe.createTimeIntegrator(fe.BDF2, nl, sys_, sol, 0.0, steps * dt, steps, guess=guess)
    return sys_, ti.makeSteps(steps)


def main(argv=None):
    from .cavity import summarize
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--re", type=float, default=100.0)
    ap.add_argument("--dt", type=float, default=0.01)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--guess", default="extrapolate", choices=["previous", "extrapolate"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--summary-from", type=int, default=3)
    args = ap.parse_args(argv)
    sys_, stats = run(args.n, args.re, args.dt, args.steps, args.guess, args.precision)
    print(json.dumps({"case": f"cube_re{args.re:g}_{args.n}^3_dt{args.dt:g}", "guess": args.guess,
                      "precision": args.precision, "summary": summarize(stats, args.summary_from),
                      "phase_ms_total": sys_.times(), "steps": stats}))


if __name__ == "__main__":
    main()
