"""Device assembly and solves on tetrahedra, through the C ABI.

* Scalar P2 (feSysElm_Diffusion<3> + feSysElm_Source on feSpaceTetPn(2)),
  against the reference library's run on the same msh file
  (tests/golden/diffusion3d_p2_4.npz): FP64 matrix and residual within
  1e-12 relative to their max norms, the FP32 matrix within 1e-5, the Newton
  solution within 1e-8; both creation routes, each with the reference's own
  tabulated rule values (its 13-decimal tetrahedral tables differ from the
  exact rules of this package by ~3e-12 relative).
* Taylor-Hood P2-P1 on tetrahedra (the reference instantiates these forms in
  2D only): residual and Jacobian against the oracle's dimension-generic
  restatement (oracle.taylor_hood, pinned on triangles against the
  reference to 1e-12 and checked on tetrahedra by finite differences and a
  manufactured solution), with every form present (transient mass with
  c0 != 0 and a nonzero u-dot, convection, stress, divergence, body force).
"""
import numpy as np
import pytest

import feng_gb300 as fe
from conftest import GOLDEN
from gpu_util import TablesSystem
from helpers import rel_err

from oracle.oracle import taylor_hood  # noqa: E402

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_FP32 = 1e-5
TOL_SOL = 1e-8


def _golden():
    with np.load(GOLDEN / "diffusion3d_p2_4.npz") as z:
        return {k: z[k] for k in z.files}


def _sin3(x, y, z):
    return (np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z),)


def _diffusion_forms(mesh):
    u = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 2, "U", "Domaine", 4)
    uB = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 2, "U", "Bord", 4, _sin3)
    num = fe.feMetaNumber(mesh, [uB, u], [uB])
    forms = [fe.createBilinearForm([u], fe.feSysElm_Diffusion(1.0)),
             fe.createBilinearForm([u], fe.feSysElm_Source(fe.api.SRC_SIN3, (-3 * np.pi ** 2,)))]
    return num, forms


def _system(route, g, precision="fp64", precond="ilu0", krylov="cg"):
    mesh = fe.Mesh3DP1.generate_cube(int(g["n"]), jitter=float(g["jitter"]), seed=int(g["seed"]))
    num, forms = _diffusion_forms(mesh)
    opts = fe.LinearSolverOptions(krylov=krylov, precond=precond, precision=precision, rel_tol=1e-12)
    if route == "tables":
        xyz = np.stack([g["x"], g["y"], g["z"]], 1)[g["tet"]].reshape(-1, 12)
        return TablesSystem(dict(g, xyz=xyz, quad_rule=g["quad"]), forms, opts)
    return fe.createLinearSystem(fe.CUDA, forms, num, opts, rule=g["quad"])


@pytest.mark.parametrize("route", ["standalone", "tables"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tet_p2_assembly_matches_reference(route, precision):
    g = _golden()
    sys_ = _system(route, g, precision, krylov="fgmres")
    sys_.setSolution(g["u0"])
    sys_.setToZero()
    sys_.assembleResiduals()
    sys_.assembleMatrices()
    sys_.synchronize()
    assert rel_err(sys_.getRHS(), g["rhs0"]) <= TOL_FP64
    assert rel_err(sys_.getMatrix(), g["values0"]) <= (TOL_FP64 if precision == "fp64" else TOL_FP32)


@pytest.mark.parametrize("route,precond", [("standalone", "ilu0"), ("standalone", "amg"), ("tables", "ilu0")])
def test_tet_p2_newton_matches_reference_solution(route, precond):
    g = _golden()
    sys_ = _system(route, g, "fp64", precond=precond)
    n = int(g["nInc"])
    sys_.setSolution(np.concatenate([np.zeros(n), g["usol"][n:]]))
    st = fe.solveNewtonRaphson(sys_, None, fe.feNLSolverOptions(tolResidual=1e-12, tolCorrection=1e-14, maxIter=10))
    assert st["return"] == 0, st
    assert rel_err(sys_.getSolution(), g["usol"]) <= TOL_SOL


def _th_case(n=3, seed=4):
    mesh = fe.Mesh3DP1.generate_cube(n, jitter=0.05, seed=seed)
    u = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 5)
    uB = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 5)
    p = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "Domaine", 5)
    num = fe.feMetaNumber(mesh, [u, uB, p], [uB])
    forms = [fe.createBilinearForm([u], fe.feSysElm_TransientVectorMass(1.3)),
             fe.createBilinearForm([u], fe.feSysElm_VectorConvectiveAcceleration(0.9)),
             fe.createBilinearForm([p, u], fe.feSysElm_MixedDivergence(1.1)),
             fe.createBilinearForm([u, p], fe.feSysElm_DivergenceNewtonianStress(-1.0, 0.02)),
             fe.createBilinearForm([u], fe.feSysElm_VectorSource(fe.api.SRC_SIN3_BODY, (2.5,)))]
    return mesh, num, forms


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tet_taylor_hood_matches_oracle(precision):
    mesh, num, forms = _th_case()
    sys_ = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond="ilu0", precision=precision))
    st = num.setup(0)
    a = mesh.arrays()
    xyz = np.stack([a["x"], a["y"], a["z"]], 1)[a["tet"]]
    rule = fe.api.tet_quadrature_rule(5)
    quad = np.stack([rule[0], rule[1], rule[2], rule[3]], 1)
    rng = np.random.default_rng(7)
    u = rng.uniform(-1, 1, sys_.nDofs)
    ud = rng.uniform(-1, 1, sys_.nDofs)
    c0 = 1.7
    sys_.setSolution(u, ud)
    sys_.setTime(0.0, c0)
    sys_.setToZero()
    sys_.assembleResiduals()
    sys_.assembleMatrices()
    sys_.synchronize()
    ia, ja = st.pattern()
    vals, rhs = taylor_hood(st.elementDofs(), xyz, quad, u, sys_.nInc, ia, ja, conv=0.9, sigma=-1.0, mu=0.02,
                            divu=1.1, mass=1.3, udot=ud, c0=c0,
                            source=lambda x, y, z: (2.5 * np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z),
                                                    0.0 * x, 0.0 * x))
    assert rel_err(sys_.getRHS(), rhs) <= TOL_FP64
    assert rel_err(sys_.getMatrix(), vals) <= (TOL_FP64 if precision == "fp64" else TOL_FP32)
    # the FP32 Jacobian is assembled row-owned (warp per velocity node or
    # pressure row), the FP64 one by the colored scatter; a second assembly
    # after setToZero overwrites the values, it does not add to them
    assert sys_.jacobianRoute == (1 if precision == "mixed" else 0)
    sys_.setToZero()
    sys_.assembleMatrices()
    sys_.synchronize()
    assert rel_err(sys_.getMatrix(), vals) <= (TOL_FP64 if precision == "fp64" else TOL_FP32)


@pytest.mark.parametrize("n", [4, 6])
def test_tet_bdf2_three_component_multigrid(n):
    """Unsteady Navier-Stokes in the cube on tetrahedra (config C5's case at a
    small size): BDF2 steps from rest with the saddle-point multigrid on the
    three velocity components, plain FP64 and mixed precision.  Both reach
    the relative residual stop at every step in a bounded number of Krylov
    iterations and give the same flow (the pressure up to its constant)."""
    from feng_gb300 import cube
    out = {}
    for prec, guess in (("fp64", "previous"), ("mixed", "extrapolate")):
        sys_, stats = cube.run(n, 100.0, 0.01, 3, guess, prec, rel=1e-10)
        assert all(s["status"] == 0 for s in stats), stats
        assert all(s["krylov_iterations"] <= 150 * max(1, s["newton_iterations"]) for s in stats), stats
        out[prec] = (sys_, sys_.getSolution())
    sys_, uf = out["fp64"]
    _, um = out["mixed"]
    x, y, fld, comp = sys_.dofInfo()
    vel = np.arange(sys_.nDofs)[fld == 0]
    prs = np.arange(sys_.nDofs)[fld == 1]
    assert np.max(np.abs(uf[vel])) > 1e-6          # the body force moved the fluid
    assert np.max(np.abs(um[vel] - uf[vel])) <= 1e-6 * np.max(np.abs(uf[vel]))
    pf, pm = uf[prs] - uf[prs].mean(), um[prs] - um[prs].mean()
    assert np.max(np.abs(pm - pf)) <= 1e-5 * np.max(np.abs(pf))
