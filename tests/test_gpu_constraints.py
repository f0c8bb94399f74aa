"""Device constraints of essential vector components and periodic DOFs
against the oracle restatement of the MKL backend
(feLinearSystemMklPardiso.cpp:994-1149), on the assembled Kovasznay Jacobian
of the golden fixture: bit-exact (assignments only), FP64 and FP32
matrices; and a Newton solve that keeps constrained components fixed."""
import numpy as np
import pytest

import feng_gb300 as fe
from conftest import load_golden
from helpers import golden_mesh, problem_spaces
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _system(precision):
    g = load_golden("kovasznay_th_8")
    num, forms = problem_spaces("ns_kovasznay", golden_mesh(g), 40.0)
    sys = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond="ilu0", precision=precision))
    sys.setSolution(g["u0"])
    return g, sys


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_constraints_match_oracle(precision):
    g, sys = _system(precision)
    ia, ja = g["ia"], g["ja"]
    n = len(ia) - 1
    rng = np.random.default_rng(8)
    rows = rng.choice(n, 30, replace=False)
    master = rng.choice(n, 5, replace=False)
    slave = (master + 11) % n
    sys.setConstrainedRows(rows)
    sys.setPeriodicPairs(master, slave)
    sys.setToZero()
    sys.assembleResiduals()
    sys.assembleMatrices()
    v0, r0 = sys.getMatrix(), sys.getRHS()
    sys.constrainEssentialComponents()
    sys.applyPeriodicity()
    v1, r1 = sys.getMatrix(), sys.getRHS()
    ve, re = orc.constrain(ia, ja, v0, r0, rows, master, slave)
    np.testing.assert_array_equal(v1, ve)
    np.testing.assert_array_equal(r1, re)
    # idempotent: a second application changes nothing
    sys.constrainEssentialComponents()
    sys.applyPeriodicity()
    np.testing.assert_array_equal(sys.getMatrix(), ve)


def test_newton_keeps_constrained_components():
    g, sys = _system("fp64")
    x, y, fld, comp = sys.dofInfo()
    # constrain the x velocity component of the first 10 unknown velocity DOFs
    rows = [d for d in range(sys.nInc) if fld[d] == 0 and comp[d] == 0][:10]
    sys.setConstrainedRows(rows)
    u0 = g["u0"].copy()
    sys.setSolution(u0)
    st = fe.solveNewtonRaphson(sys, None, fe.feNLSolverOptions(tolResidual=0.0, tolCorrection=0.0, maxIter=10,
                                                                 relResidual=1e-8))
    u = sys.getSolution()
    np.testing.assert_array_equal(u[rows], u0[rows])
    assert st["iterations"] >= 1
