"""Device error norms (fe_cuda_l2_error) and the device Newton solve against
the reference's golden convergence outputs: P2 diffusion
(tests/withLinearSolver/scalarFE_diffusion.output) and Taylor-Hood
Navier-Stokes MMS (navier_stokes_MMS.output, divergence formulation) on the
reference's meshes.  The errors must print as the golden files do (7
significant digits, as the reference's compareOutputFiles), and the device
norm of the device solution must equal the oracle's norm of the same
solution to 1e-12 relative."""
import pytest

import feng_gb300 as fe
from helpers import convergence_case, element_xy, reference_l2

from oracle.oracle import l2_error

pytestmark = pytest.mark.gpu


def printed(v):
    return f"{float(v):.6e}"


def _solve(key, i, precision="fp64"):
    g = reference_l2()
    mesh, num, forms, spaces, fcts = convergence_case(g, key, i)
    opts = fe.LinearSolverOptions(precond="ilu0", rel_tol=1e-12, precision=precision, max_iter=4000)
    sys_ = fe.createLinearSystem(fe.CUDA, forms, num, opts)
    sol = fe.feSolution(sys_)
    sol.initializeEssentialBC()
    # NLoptions of the reference's convergence drivers (scalarFE.cpp:765)
    st = fe.solveNewtonRaphson(sys_, sol, fe.feNLSolverOptions(1e-10, 1e-10, 1e4, 20, 4, 1e-1))
    assert st["return"] == 0, st
    return g, mesh, num, sys_, sol, spaces, fcts


@pytest.mark.parametrize("i", [1, 2, 3, 4])
def test_diffusion_p2_errors_match_reference_output(i):
    g, mesh, num, sys_, sol, (u,), (fct,) = _solve("diff", i)
    e = fe.createNorm(fe.L2_ERROR, [u], sol, fct).compute()
    assert printed(e) == printed(g["diff_err_u"][i - 1])
    st = num.setup(256)
    eo = l2_error(num.elem_type, st.elementDofs(), element_xy(mesh), sys_.getSolution(), fe.api.quadrature_rule(8),
                  fct, 0)
    assert e == pytest.approx(eo, rel=1e-12)


@pytest.mark.parametrize("i", [1, 2, 3, 4])
def test_navier_stokes_mms_errors_match_reference_output(i):
    g, mesh, num, sys_, sol, (u, p), (fu, fp) = _solve("ns", i)
    eu = fe.createNorm(fe.VECTOR_L2_ERROR, [u], sol, None, fu).compute()
    ep = fe.createNorm(fe.L2_ERROR, [p], sol, fp).compute()
    assert printed(eu) == printed(g["ns_err_u"][i - 1])
    assert printed(ep) == printed(g["ns_err_p"][i - 1])
    st = num.setup(256)
    adr, xy, usol, q = st.elementDofs(), element_xy(mesh), sys_.getSolution(), fe.api.quadrature_rule(8)
    assert eu == pytest.approx(l2_error(num.elem_type, adr, xy, usol, q, fu, 0), rel=1e-12)
    assert ep == pytest.approx(l2_error(num.elem_type, adr, xy, usol, q, fp, 1), rel=1e-12)


def test_mixed_precision_solution_has_the_same_errors():
    """The mixed path (FP32 Jacobian and Krylov, FP64 residual) converges to
    the same discrete solution: errors print the same on the finest mesh."""
    g, mesh, num, sys_, sol, (u, p), (fu, fp) = _solve("ns", 4, precision="mixed")
    assert printed(fe.createNorm(fe.VECTOR_L2_ERROR, [u], sol, None, fu).compute()) == printed(g["ns_err_u"][3])
    assert printed(fe.createNorm(fe.L2_ERROR, [p], sol, fp).compute()) == printed(g["ns_err_p"][3])


def test_norm_argument_errors():
    g = reference_l2()
    mesh, num, forms, (u, p), (fu, fp) = convergence_case(g, "ns", 1)
    sys_ = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond="ilu0"))
    sol = fe.feSolution(sys_)
    with pytest.raises(ValueError):
        fe.createNorm(fe.L2_ERROR, [u], sol, fu)          # vector space needs VECTOR_L2_ERROR
    with pytest.raises(ValueError):
        fe.createNorm(fe.VECTOR_L2_ERROR, [u], sol)       # no exact solution
    nq = fe.createNorm(fe.L2_ERROR, [p], sol, fp).points()[0].shape
    assert nq == (len(g["ns1_tri"]), 16)
