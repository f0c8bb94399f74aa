"""Parity of the CUDA path with the reference feNG library (golden fixtures
from tests/golden/make_golden.py), through the C ABI.

Tolerances: assembled FP64 matrix and residual 1e-12 relative to their max
norm (the mixed path's double-float residual too); FP32 matrix 1e-5
relative; converged solutions 1e-8 relative."""
import numpy as np
import pytest

import feng_gb300 as fe
from conftest import golden_names, load_golden
from gpu_util import TablesSystem
from helpers import golden_mesh, problem_spaces, rel_err

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_FP32 = 1e-5
TOL_SOL = 1e-8


def _assemble(sys, u0):
    sys.setSolution(u0)
    sys.setToZero()
    sys.assembleResiduals()
    sys.assembleMatrices()
    sys.synchronize()
    return sys.getMatrix(), sys.getRHS()


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("route", ["tables", "standalone"])
def test_assembly_fp64_matches_reference(name, route):
    g = load_golden(name)
    num, forms = problem_spaces(str(g["problem"]), golden_mesh(g), float(g["re"]))
    opts = fe.LinearSolverOptions(precond="ilu0")
    sys = TablesSystem(g, forms, opts) if route == "tables" else fe.createLinearSystem(fe.CUDA, forms, num, opts)
    vals, rhs = _assemble(sys, g["u0"])
    assert rel_err(vals, g["values0"]) <= TOL_FP64
    assert rel_err(rhs, g["rhs0"]) <= TOL_FP64


@pytest.mark.parametrize("name", golden_names())
def test_assembly_fp32_matrix(name):
    g = load_golden(name)
    num, forms = problem_spaces(str(g["problem"]), golden_mesh(g), float(g["re"]))
    sys = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond="ilu0", precision="mixed"))
    vals, rhs = _assemble(sys, g["u0"])
    assert rel_err(vals, g["values0"]) <= TOL_FP32
    assert rel_err(rhs, g["rhs0"]) <= TOL_FP64  # the residual: double-float, FP64-class


def test_double_float_residual_with_mass_matches_fp64():
    """The mixed path's residual (double-float, k_residual_th_df) against the
    FP64 kernel on the lid-driven cavity forms (transient mass with a
    nonzero u-dot, convection, stress, divergence) at a random state."""
    from helpers import cavity_spaces
    mesh = fe.Mesh2DP1.generate_square(8, jitter=0.1, seed=3)
    num, forms = cavity_spaces(mesh, 100.0)
    rng = np.random.default_rng(5)
    u = ud = None
    res = {}
    for prec in ("fp64", "mixed"):
        sys = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond="ilu0", precision=prec))
        if u is None:
            u = rng.uniform(-1, 1, sys.nDofs)
            ud = rng.uniform(-1, 1, sys.nDofs)
        sys.setSolution(u, ud)
        sys.setToZero()
        sys.assembleResiduals()
        sys.synchronize()
        res[prec] = sys.getRHS()
    assert rel_err(res["mixed"], res["fp64"]) <= TOL_FP64


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_newton_converges_to_reference_solution(name, precision):
    g = load_golden(name)
    num, forms = problem_spaces(str(g["problem"]), golden_mesh(g), float(g["re"]))
    krylov = "cg" if str(g["problem"]) == "diffusion" and precision == "fp64" else "fgmres"
    opts = fe.LinearSolverOptions(krylov=krylov, precond="ilu0", precision=precision, rel_tol=1e-12)
    sys = fe.createLinearSystem(fe.CUDA, forms, num, opts)
    sol = fe.feSolution(sys)
    sol.initializeEssentialBC()
    st = fe.solveNewtonRaphson(sys, sol, fe.feNLSolverOptions(tolResidual=1e-12, tolCorrection=1e-14, maxIter=30))
    assert st["return"] == 0, st
    assert rel_err(sol.u, g["usol"]) <= TOL_SOL


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_newton_multigrid_preconditioner(name, precision):
    g = load_golden(name)
    num, forms = problem_spaces(str(g["problem"]), golden_mesh(g), float(g["re"]))
    krylov = "cg" if str(g["problem"]) == "diffusion" and precision == "fp64" else "fgmres"
    opts = fe.LinearSolverOptions(krylov=krylov, precond="amg", precision=precision, rel_tol=1e-12)
    sys = fe.createLinearSystem(fe.CUDA, forms, num, opts)
    sol = fe.feSolution(sys)
    sol.initializeEssentialBC()
    st = fe.solveNewtonRaphson(sys, sol, fe.feNLSolverOptions(tolResidual=1e-12, tolCorrection=1e-14, maxIter=30))
    assert st["return"] == 0, st
    assert rel_err(sol.u, g["usol"]) <= TOL_SOL


def test_kovasznay_block_jacobi_fgmres():
    g = load_golden("kovasznay_th_8")
    num, forms = problem_spaces("ns_kovasznay", golden_mesh(g), 40.0)
    sys = fe.createLinearSystem(fe.CUDA, forms, num,
                                fe.LinearSolverOptions(precond="bjacobi-ilu0", pc_block_rows=64, rel_tol=1e-10))
    sol = fe.feSolution(sys)
    sol.initializeEssentialBC()
    st = fe.solveNewtonRaphson(sys, sol, fe.feNLSolverOptions(tolResidual=1e-12, maxIter=30))
    assert st["return"] == 0
    assert rel_err(sol.u, g["usol"]) <= TOL_SOL


def test_mixed_krylov_at_large_size_matches_fp64():
    """Mixed FGMRES on more than 4 M rows' worth of Gram-Schmidt chunks
    (1024 blocks of partial sums are exceeded, so the dot pass loops over
    chunks): a Kovasznay 400 x 400 Newton solve converges like the FP64 one."""
    from feng_gb300 import kovasznay
    _, num, forms = kovasznay.build(400, 40.0)
    out = {}
    for prec in ("fp64", "mixed"):
        sys, _ = kovasznay.make_system(num, forms, prec)
        st = fe.solveNewtonRaphson(sys, None, kovasznay.newton_options(prec))
        assert st["return"] == 0, (prec, st)
        assert st["residual"] <= 1e-8 * st["residual0"]
        out[prec] = sys.getSolution()
    # both stop at ||R|| <= 1e-8 ||R0||; at this size that bounds the
    # difference of the two solutions near 1e-5 relative (max norm)
    assert rel_err(out["mixed"], out["fp64"]) <= 1e-5
