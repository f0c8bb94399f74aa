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


def reference_l2():
    """Meshes and golden L2 errors of the reference's convergence tests
    (tests/golden/norms/make_reference_norms.py)."""
    from pathlib import Path
    p = Path(__file__).resolve().parent / "golden" / "norms" / "reference_l2.npz"
    with np.load(p) as z:
        return {k: z[k] for k in z.files}


def convergence_case(g, key, i):
    """One mesh of the reference's convergence tests with its spaces and
    forms: key "diff" = P2 diffusion of u = sin(pi x) sin(pi y) on
    data/mmsMeshes/square<i>.msh (tests/withLinearSolver/scalarFE.cpp:37-56,
    802), key "ns" = Taylor-Hood Navier-Stokes MMS, divergence formulation,
    velocity and pressure essential on "Bord", on data/square<i>.msh
    (tests/withLinearSolver/navier_stokes.cpp:63-92, 355).  Quadrature degree
    8.  Returns (mesh, numbering, forms, norm spaces, exact functions)."""
    mesh = fe.Mesh2DP1.from_arrays(g[f"{key}{i}_x"], g[f"{key}{i}_y"], g[f"{key}{i}_tri"], g[f"{key}{i}_bnd"],
                                   int(g[f"{key}{i}_point"]))
    if key == "diff":
        uB = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 2, "U", "Bord", 8, exact.sin_sin)
        u = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 2, "U", "Domaine", 8, exact.zero_scalar)
        num = fe.feMetaNumber(mesh, [uB, u], [uB])
        forms = [fe.createBilinearForm([u], fe.feSysElm_Diffusion(1.0)),
                 fe.createBilinearForm([u], fe.feSysElm_Source(fe.api.SRC_SIN_SIN, (-2 * np.pi ** 2,)))]
        return mesh, num, forms, [u], [exact.sin_sin]
    u = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 8, exact.ns_mms_velocity)
    uB = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 8, exact.ns_mms_velocity)
    p = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "Domaine", 8, exact.ns_mms_pressure)
    pB = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "Bord", 8, exact.ns_mms_pressure)
    num = fe.feMetaNumber(mesh, [u, uB, p, pB], [uB, pB])
    forms = [fe.createBilinearForm([u], fe.feSysElm_VectorConvectiveAcceleration(-1.0)),
             fe.createBilinearForm([p, u], fe.feSysElm_MixedDivergence(1.0)),
             fe.createBilinearForm([u], fe.feSysElm_VectorSource(fe.api.SRC_NS_MMS_POLY)),
             fe.createBilinearForm([u, p], fe.feSysElm_DivergenceNewtonianStress(1.0, 1.0))]
    return mesh, num, forms, [u, p], [exact.ns_mms_velocity, exact.ns_mms_pressure]


def poiseuille_case(g, stokes):
    """The Poiseuille tests of the reference on data/poiseuille0.msh,
    divergence formulation, P2-P1, quadrature degree 8
    (tests/withLinearSolver/navier_stokes.cpp:194-290, stokes.cpp:183-279):
    velocity essential on "NoSlip" and "Inlet" (one space here: the exact
    profile vanishes on the walls), the vertical velocity constrained on
    "Outlet" (setEssentialComponent(1)), pressure free.  Navier-Stokes:
    convective acceleration +1, divergence +1, Newtonian stress -1 with
    viscosity 1; Stokes: divergence +1, stress +1.  Returns (mesh, numbering,
    forms, outlet rows, exact functions)."""
    uex, pex = exact.poiseuille_velocity(), exact.poiseuille_pressure()
    mesh = fe.Mesh2DP1.from_arrays(g["pois_x"], g["pois_y"], g["pois_tri"], g["pois_bnd"], -1)
    u = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 8, exact.zero_vector)
    uB = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 8, uex)
    p = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "Domaine", 8, exact.zero_scalar)
    num = fe.feMetaNumber(mesh, [uB, u, p], [uB])
    forms = [fe.createBilinearForm([p, u], fe.feSysElm_MixedDivergence(1.0))]
    if stokes:
        forms.append(fe.createBilinearForm([u, p], fe.feSysElm_DivergenceNewtonianStress(1.0, 1.0)))
    else:
        forms.insert(0, fe.createBilinearForm([u], fe.feSysElm_VectorConvectiveAcceleration(1.0)))
        forms.append(fe.createBilinearForm([u, p], fe.feSysElm_DivergenceNewtonianStress(-1.0, 1.0)))
    return mesh, num, forms, outlet_rows(mesh, num, g["pois_outlet"], 1), [uex, pex]


def outlet_rows(mesh, num, lines, comp):
    """Unknowns of velocity component `comp` on the given boundary lines (the
    rows constrainEssentialComponents collects from the addressing vectors of
    a space on those lines, src/feLinearSystemMklPardiso.cpp:994-1030): the
    P2 vertex and edge DOFs of each line, taken from the triangle that holds
    it (local node k of a Taylor-Hood element, component c, at 2k+c; edge
    nodes 3-5 join local vertices (0,1), (1,2), (2,0))."""
    st = num.setup(256)
    tri, adr = mesh.arrays()["tri"], st.elementDofs()
    rows = set()
    for a, b in np.asarray(lines).reshape(-1, 2):
        t = int(np.flatnonzero((tri == a).any(1) & (tri == b).any(1))[0])
        la, lb = int(np.flatnonzero(tri[t] == a)[0]), int(np.flatnonzero(tri[t] == b)[0])
        le = 3 + next(k for k in range(3) if {k, (k + 1) % 3} == {la, lb})
        for node in (la, lb, le):
            d = int(adr[t, 2 * node + comp])
            if d < st.nInc:
                rows.add(d)
    return np.array(sorted(rows), np.int64)


def essential_state(num, fcts_by_field):
    """Zero unknowns and the exact values on the essential DOFs (nodewise,
    as feSolution::initializeEssentialBC)."""
    st = num.setup(256)
    x, y, fld, comp, _ = st.dofInfo()
    u = np.zeros(st.nDofs)
    ess = np.arange(st.nInc, st.nDofs)
    for f, fct in enumerate(fcts_by_field):
        sel = ess[fld[ess] == f]
        vals = fct(x[sel], y[sel])
        for c in range(len(vals)):
            m = comp[sel] == c
            u[sel[m]] = np.broadcast_to(vals[c], sel.shape)[m]
    return u


def element_xy(mesh):
    arr = mesh.arrays()
    tri = arr["tri"]
    return np.stack([arr["x"][tri[:, 0]], arr["y"][tri[:, 0]], arr["x"][tri[:, 1]], arr["y"][tri[:, 1]],
                     arr["x"][tri[:, 2]], arr["y"][tri[:, 2]]], 1)
