"""BDF2 time integration on the device against the reference's own
BDF2Integrator (golden fixture cavity_bdf2_8: lid-driven cavity from rest,
BDF1 starter, Eigen LU Newton solves to ||R||inf <= 1e-11), and what the
learned Newton initial guess gains over plain extrapolation.

Tolerance of the solution parity: 1e-8 relative (max norm), as for the
steady Newton solutions."""
import numpy as np
import pytest

import feng_gb300 as fe
from conftest import golden_names, load_golden
from helpers import cavity_spaces, golden_mesh, rel_err

pytestmark = pytest.mark.gpu

TOL_SOL = 1e-8


def _cavity_system(mesh, re, precision="fp64", precond="ilu0", rel_tol=1e-12):
    num, forms = cavity_spaces(mesh, re)
    opts = fe.LinearSolverOptions(precond=precond, rel_tol=rel_tol, max_iter=2000, precision=precision)
    sys = fe.createLinearSystem(fe.CUDA, forms, num, opts)
    sol = fe.feSolution(sys)
    sol.initializeEssentialBC()
    return sys, sol


def _tight():
    return fe.feNLSolverOptions(tolResidual=1e-11, tolCorrection=1e-13, tolDivergence=1e12, maxIter=30)


@pytest.mark.parametrize("name", golden_names(transient=True))
@pytest.mark.parametrize("guess", ["previous", "extrapolate"])
def test_bdf2_matches_reference_integrator(name, guess):
    g = load_golden(name)
    re, dt, steps = float(g["re"]), float(g["dt"]), int(g["steps"])
    sys, sol = _cavity_system(golden_mesh(g), re)
    ti = fe.createTimeIntegrator(fe.BDF2, _tight(), sys, sol, 0.0, steps * dt, steps, guess=guess)
    stats = ti.makeSteps(steps)
    assert all(s["status"] == 0 for s in stats), stats
    assert [s["step"] for s in stats] == list(range(1, steps + 1))
    assert stats[-1]["t"] == pytest.approx(steps * dt, rel=1e-12)
    u = sys.getSolution()
    assert rel_err(u, g["usol"]) <= TOL_SOL
    if guess == "extrapolate":
        # Once the impulsive start is over (step 4 on) the extrapolation
        # starts Newton closer to the solution than u^n does.
        assert all(s["guess_used"] == 1 for s in stats[1:])
        assert max(s["residual_guess"] / s["residual_ref"] for s in stats[3:]) < 0.5


def _run(guess, n=24, re=100.0, dt=0.01, steps=40, **kw):
    mesh = fe.Mesh2DP1.generate_square(n, 0.0, 1.0, 0.0, 1.0, jitter=0.1, seed=7)
    sys, sol = _cavity_system(mesh, re, precision="mixed", precond="amg", rel_tol=1e-8)
    nl = fe.feNLSolverOptions(tolResidual=0.0, tolCorrection=0.0, tolDivergence=1e12, maxIter=30,
                              relResidual=1e-8, linearRtolMin=1e-6)
    ti = fe.createTimeIntegrator(fe.BDF2, nl, sys, sol, 0.0, steps * dt, steps, guess=guess, **kw)
    stats = ti.makeSteps(steps)
    return sys.getSolution(), stats


def test_learned_guess_gain_over_extrapolation():
    """Same cavity run with the extrapolated and with the learned guess
    (trained from step 5, used from step 10): both reach the same solution,
    and over steps 20-40 the learned guess starts Newton closer to the
    solution and needs no more Newton iterations."""
    kw = dict(trainFrom=5, useFrom=10, trainIters=16, batch=4096, lr=2e-3, seed=3)
    ue, se = _run("extrapolate")
    ul, sl = _run("learned", **kw)
    assert all(s["status"] == 0 for s in se + sl)
    assert rel_err(ul, ue) <= 1e-6          # both converged to 1e-8 relative residual
    late = slice(19, 40)
    r_e = np.array([s["residual_guess"] / s["residual_ref"] for s in se[late]])
    r_l = np.array([s["residual_guess"] / s["residual_ref"] for s in sl[late]])
    used = sum(s["guess_used"] == 2 for s in sl[late])
    newton_e = sum(s["newton_iterations"] for s in se[late])
    newton_l = sum(s["newton_iterations"] for s in sl[late])
    krylov_e = sum(s["krylov_iterations"] for s in se[late])
    krylov_l = sum(s["krylov_iterations"] for s in sl[late])
    print(f"\nlearned guess over steps 20-40: used {used}/21, initial residual ratio "
          f"{np.exp(np.mean(np.log(r_l))):.3e} vs extrapolation {np.exp(np.mean(np.log(r_e))):.3e}; "
          f"Newton {newton_l} vs {newton_e}, Krylov {krylov_l} vs {krylov_e}; "
          f"train loss {sl[-1]['train_loss']:.3e}")
    # The fallback makes the learned run's start never worse than extrapolation.
    assert all(s["residual_guess"] <= s["residual_extrap"] * (1 + 1e-12) for s in sl[late] if s["guess_used"] == 2)
    assert used >= 10
    assert np.exp(np.mean(np.log(r_l))) < 0.7 * np.exp(np.mean(np.log(r_e)))
    assert newton_l <= newton_e
