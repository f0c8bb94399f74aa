"""The level-scheduled ILU(0) preconditioner on the device against the
oracle's serial ILU(0) (Saad, Alg. 10.4, oracle/fe_oracle.c), through the
C ABI (fe_cuda_apply_preconditioner).

The device factorisation applies each row's updates in the serial order, so
its factors equal the serial ones; the triangular solves sum each row in a
different order.  Tolerance of z = (LU)^-1 r: 1e-12 relative to max |z| in
FP64, 1e-5 with the FP32 factors of the mixed path.  Cases: the 64 x 64 P2
diffusion system of the CPU-runnable configuration as one block (254
levels in its L and in its U part), and a Taylor-Hood Jacobian in
block-Jacobi form (the blocks of the set-up's partition)."""
import numpy as np
import pytest

import feng_gb300 as fe
from conftest import load_golden
from helpers import golden_mesh, problem_spaces

from oracle.oracle import OracleProblem  # noqa: E402

pytestmark = pytest.mark.gpu


def _oracle_ilu(g, vals, r, blocks=None):
    from feng_gb300.api import quadrature_rule
    nloc = g["adr"].size // len(g["tri"])
    op = OracleProblem(1 if nloc == 6 else 2, g["adr"], np.zeros((len(g["tri"]), 6)), int(g["nInc"]),
                       int(g["nDofs"]), g["color_offsets"], g["color_elements"], g["ia"], g["ja"],
                       quadrature_rule(int(g["quad_degree"])), [])
    return op.apply_ilu(vals, r, blocks)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ilu0_single_block_matches_serial(precision):
    g = load_golden("diffusion_p2_64")
    num, forms = problem_spaces("diffusion", golden_mesh(g))
    sys_ = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(krylov="fgmres", precond="ilu0",
                                                                            precision=precision))
    sys_.setSolution(g["u0"])
    sys_.setToZero()
    sys_.assembleMatrices()
    r = np.random.default_rng(3).uniform(-1, 1, sys_.nInc)
    z = sys_.applyPreconditioner(r)
    zo = _oracle_ilu(g, sys_.getMatrix(), r)
    tol = 1e-12 if precision == "fp64" else 1e-5
    assert np.max(np.abs(z - zo)) <= tol * np.max(np.abs(zo))


def test_ilu0_block_jacobi_matches_serial():
    g = load_golden("kovasznay_th_8")
    num, forms = problem_spaces("ns_kovasznay", golden_mesh(g), 40.0)
    opts = fe.LinearSolverOptions(precond="bjacobi-ilu0", pc_block_rows=64)
    sys_ = fe.createLinearSystem(fe.CUDA, forms, num, opts)
    sys_.setSolution(g["u0"])
    sys_.setToZero()
    sys_.assembleMatrices()
    r = np.random.default_rng(4).uniform(-1, 1, sys_.nInc)
    z = sys_.applyPreconditioner(r)
    zo = _oracle_ilu(g, sys_.getMatrix(), r, num.setup(64).blocks())
    assert np.max(np.abs(z - zo)) <= 1e-12 * np.max(np.abs(zo))
