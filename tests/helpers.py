"""Problem builders shared by the tests, mirroring the reference test drivers
(tests/withLinearSolver/scalarFE.cpp:35-60, navier_stokes.cpp:64-100)."""
import numpy as np

import feng_gb300 as fe
from feng_gb300 import exact


def problem_spaces(problem, mesh, re=40.0):
    """Returns (numbering, forms) of one benchmark problem."""
    if problem == "diffusion":
        u = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 2, "U", "Domaine", 4, exact.zero_scalar)
        uB = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 2, "U", "Bord", 4, exact.sin_sin)
        num = fe.feMetaNumber(mesh, [uB, u], [uB])
        forms = [fe.createBilinearForm([u], fe.feSysElm_Diffusion(1.0)),
                 fe.createBilinearForm([u], fe.feSysElm_Source(fe.api.SRC_SIN_SIN, (-2 * np.pi ** 2,)))]
        return num, forms
    if problem == "ns_cavity_bdf2":
        return cavity_spaces(mesh, re)
    kov = problem == "ns_kovasznay"
    uex = exact.kovasznay_velocity(re) if kov else exact.ns_mms_velocity
    pex = exact.kovasznay_pressure(re) if kov else exact.ns_mms_pressure
    u = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 8, uex)
    uB = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 8, uex)
    p = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "Domaine", 8, pex)
    pP = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "PointPression", 8, pex)
    num = fe.feMetaNumber(mesh, [u, uB, p, pP], [uB, pP])
    forms = [fe.createBilinearForm([u], fe.feSysElm_VectorConvectiveAcceleration(-1.0)),
             fe.createBilinearForm([p, u], fe.feSysElm_MixedDivergence(1.0)),
             fe.createBilinearForm([u, p], fe.feSysElm_DivergenceNewtonianStress(1.0, 1.0 / re if kov else 1.0))]
    if not kov:
        forms.append(fe.createBilinearForm([u], fe.feSysElm_VectorSource(fe.api.SRC_NS_MMS_POLY)))
    return num, forms


def cavity_spaces(mesh, re):
    """Lid-driven cavity with the transient forms and the sign convention of
    the reference's unsteady Navier-Stokes test
    (tests/withLinearSolver/vectorFEunsteady.cpp:560-584)."""
    lid = exact.cavity_lid()
    u = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 8, lid)
    uB = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 8, lid)
    p = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "Domaine", 8, exact.zero_scalar)
    pP = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "PointPression", 8, exact.zero_scalar)
    num = fe.feMetaNumber(mesh, [u, uB, p, pP], [uB, pP])
    forms = [fe.createBilinearForm([u], fe.feSysElm_TransientVectorMass(1.0)),
             fe.createBilinearForm([u], fe.feSysElm_VectorConvectiveAcceleration(1.0)),
             fe.createBilinearForm([p, u], fe.feSysElm_MixedDivergence(1.0)),
             fe.createBilinearForm([u, p], fe.feSysElm_DivergenceNewtonianStress(-1.0, 1.0 / re))]
    return num, forms


def golden_mesh(g):
    dom = tuple(float(v) for v in g["domain"])
    return fe.Mesh2DP1.generate_square(int(g["n"]), *dom, jitter=float(g["jitter"]), seed=int(g["seed"]))


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
