"""Failure statuses of the device path, each failure made on the host.

Where the reference exits (src/feNonLinearSolver.cpp:108-119,174-180) the
backend returns a status instead: a NaN or infinity in the state gives
FE_CUDA_NONFINITE (-7), an ILU(0) zero pivot FE_CUDA_PC_FAILED (-6), a solve
or time step that does not converge FE_CUDA_NOT_CONVERGED (-5), and a
coloring whose same-color elements share a DOF FE_CUDA_BAD_COLORING (-8).
No test here faults the GPU: the bad values are host inputs (a state, a
coefficient, an iteration limit, a coloring, the network's parameters), and
every device loop involved is bounded."""
import numpy as np
import pytest

import feng_gb300 as fe
from conftest import load_golden
from feng_gb300._lib import FeError
from gpu_util import TablesSystem
from helpers import cavity_spaces, golden_mesh, problem_spaces

pytestmark = pytest.mark.gpu

NONFINITE, PC_FAILED, NOT_CONVERGED, BAD_COLORING, INVALID_ARG = -7, -6, -5, -8, -3


def _kovasznay(precision="fp64", precond="ilu0", **kw):
    g = load_golden("kovasznay_th_8")
    num, forms = problem_spaces("ns_kovasznay", golden_mesh(g), 40.0)
    sys = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond=precond, precision=precision,
                                                                             **kw))
    return g, sys


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_nonfinite_state_gives_nonfinite_residual_norm(precision, bad):
    g, sys = _kovasznay(precision)
    u = g["u0"].copy()
    u[7] = bad
    sys.setSolution(u)
    sys.setToZero()
    sys.assembleResiduals()
    with pytest.raises(FeError) as e:
        sys.getRHSMaxNorm()
    assert e.value.status == NONFINITE


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_all_nan_residual_is_not_convergence(precision):
    """Every unknown NaN: the max-norm of the residual is NaN, not 0 (a
    max that dropped NaN operands would read 0 here and stop Newton at
    iteration 0 with success)."""
    g, sys = _kovasznay(precision)
    u = g["u0"].copy()
    u[: int(g["nInc"])] = np.nan
    sys.setSolution(u)
    with pytest.raises(FeError) as e:
        fe.solveNewtonRaphson(sys, None, fe.feNLSolverOptions(tolResidual=1e-12, maxIter=5))
    assert e.value.status == NONFINITE


def test_noalloc_max_norm_propagates_nan():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    import ctypes as C
    from feng_gb300 import _lib
    lib = _lib.load()
    x = torch.zeros(100_000, dtype=torch.float64, device="cuda:0")
    x[12345] = float("nan")
    out = C.c_double(0.0)
    assert lib.fe_cuda_max_norm_noalloc(C.c_void_p(x.data_ptr()), x.numel(), None, C.byref(out)) == 0
    assert np.isnan(out.value)


def test_zero_pivot_gives_pc_failed():
    """Tables route, P2 diffusion with a zero coefficient: every matrix entry
    (the diagonal included) is 0, so ILU(0) meets a zero pivot."""
    g = load_golden("diffusion_p2_8")
    _, forms = problem_spaces("diffusion", golden_mesh(g))
    forms = [fe.createBilinearForm(f.spaces, fe.feSysElm_Diffusion(0.0)) if f.sysElm.kind == 2 else f
             for f in forms]
    sys = TablesSystem(g, forms, fe.LinearSolverOptions(krylov="cg", precond="ilu0"))
    sys.setSolution(g["u0"])
    sys.setToZero()
    sys.assembleResiduals()
    sys.assembleMatrices()
    r = sys.solve(raise_on_failure=False)
    assert r["status"] == PC_FAILED


def test_linear_iteration_limit_gives_not_converged():
    g, sys = _kovasznay()
    sys.setSolution(g["u0"])
    sys.setToZero()
    sys.assembleResiduals()
    sys.assembleMatrices()
    sys.setTolerances(rel_tol=1e-14, max_iter=1)
    r = sys.solve(raise_on_failure=False)
    assert r["status"] == NOT_CONVERGED
    assert r["nIter"] <= 1


def test_newton_iteration_limit_gives_not_converged():
    g, sys = _kovasznay(rel_tol=1e-12)
    sol = fe.feSolution(sys)
    sol.initializeEssentialBC()
    st = fe.solveNewtonRaphson(sys, sol, fe.feNLSolverOptions(tolResidual=1e-30, tolCorrection=0.0, maxIter=1))
    assert st["return"] == NOT_CONVERGED
    assert st["iterations"] == 2  # the reference's loop runs while iter <= maxIter


def test_time_step_that_does_not_converge_is_reported():
    """A BDF2 step whose Newton solve hits its iteration limit stops the run
    with FE_CUDA_NOT_CONVERGED (it is not counted as a converged step)."""
    mesh = fe.Mesh2DP1.generate_square(8, jitter=0.1, seed=5)
    num, forms = cavity_spaces(mesh, 100.0)
    sys = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond="ilu0", rel_tol=1e-12))
    sol = fe.feSolution(sys)
    sol.initializeEssentialBC()
    nl = fe.feNLSolverOptions(tolResidual=1e-30, tolCorrection=0.0, tolDivergence=1e12, maxIter=1)
    ti = fe.createTimeIntegrator(fe.BDF2, nl, sys, sol, 0.0, 0.05, 5, guess="extrapolate")
    with pytest.raises(FeError) as e:
        ti.makeSteps(3)
    assert e.value.status == NOT_CONVERGED
    stats = fe.createTimeIntegrator(fe.BDF2, nl, sys, sol, 0.0, 0.05, 5, guess="extrapolate").makeSteps(
        3, raise_on_failure=False)
    assert len(stats) == 1 and stats[-1]["status"] == NOT_CONVERGED


def test_nan_network_loses_to_extrapolation():
    """The learned guess with every network parameter NaN: its candidate's
    residual is NaN, so the extrapolation is used and the steps converge."""
    mesh = fe.Mesh2DP1.generate_square(8, jitter=0.1, seed=5)
    num, forms = cavity_spaces(mesh, 100.0)
    sys = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond="ilu0", rel_tol=1e-12))
    sol = fe.feSolution(sys)
    sol.initializeEssentialBC()
    nl = fe.feNLSolverOptions(tolResidual=0.0, tolCorrection=0.0, tolDivergence=1e12, maxIter=30, relResidual=1e-8)
    ti = fe.createTimeIntegrator(fe.BDF2, nl, sys, sol, 0.0, 0.1, 10, guess="learned", trainFrom=3, useFrom=4,
                                 trainIters=4, batch=256)
    first = ti.makeSteps(4)
    assert all(s["status"] == 0 for s in first)
    saved = ti.getNetwork()
    assert np.all(np.isfinite(saved))
    ti.setNetwork(np.full_like(saved, np.nan))
    late = ti.makeSteps(3)
    assert all(s["status"] == 0 for s in late), late
    assert all(s["guess_used"] == 1 for s in late), [s["guess_used"] for s in late]
    assert all(np.isfinite(s["residual"]) for s in late)


def test_coloring_with_shared_dofs_is_refused():
    g = load_golden("diffusion_p2_8")
    _, forms = problem_spaces("diffusion", golden_mesh(g))
    one = dict(g)
    n = len(g["tri"])
    one["color_offsets"] = np.array([0, n], np.int64)       # every element in one color
    one["color_elements"] = np.arange(n, dtype=np.int32)
    with pytest.raises(FeError) as e:
        TablesSystem(one, forms, fe.LinearSolverOptions(precond="ilu0"))
    assert e.value.status == BAD_COLORING


@pytest.mark.parametrize("defect", ["element_out_of_range", "element_repeated", "offsets_decrease"])
def test_malformed_coloring_is_refused(defect):
    g = load_golden("diffusion_p2_8")
    _, forms = problem_spaces("diffusion", golden_mesh(g))
    bad = dict(g)
    el = g["color_elements"].astype(np.int32).copy()
    off = g["color_offsets"].astype(np.int64).copy()
    if defect == "element_out_of_range":
        el[3] = len(g["tri"]) + 5
    elif defect == "element_repeated":
        el[3] = el[4]
    else:
        off[1], off[2] = off[2], off[1]
    bad["color_elements"], bad["color_offsets"] = el, off
    with pytest.raises(FeError) as e:
        TablesSystem(bad, forms, fe.LinearSolverOptions(precond="ilu0"))
    assert e.value.status == BAD_COLORING


def test_dof_id_out_of_range_is_refused():
    g = load_golden("diffusion_p2_8")
    _, forms = problem_spaces("diffusion", golden_mesh(g))
    bad = dict(g)
    adr = g["adr"].astype(np.int64).copy()
    adr[10] = int(g["nDofs"]) + 3
    bad["adr"] = adr
    with pytest.raises(FeError) as e:
        TablesSystem(bad, forms, fe.LinearSolverOptions(precond="ilu0"))
    assert e.value.status == INVALID_ARG


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_correction_max_norm_on_device(precision):
    """getResidualMaxNorm reduces du on the device (the same NaN-propagating
    max as the residual norm): equal to max |du| of the downloaded
    correction."""
    g, sys = _kovasznay(precision)
    sys.setSolution(g["u0"].copy())
    sys.setToZero()
    sys.assembleResiduals()
    sys.assembleMatrices()
    sys.solve()
    du = sys.getDu()
    assert np.all(np.isfinite(du)) and np.abs(du).max() > 0
    assert sys.getResidualMaxNorm() == np.abs(du).max()
