"""The oracle's dimension-generic numpy restatement of the Taylor-Hood forms
(oracle.taylor_hood): on triangles against the reference's assembled
fixtures and the C oracle, on tetrahedra (forms the reference does not
instantiate in 3D) by a finite-difference check of the Jacobian and the
transpose relation of the divergence and pressure-gradient blocks.  Runs on
the CPU."""
import numpy as np
import pytest

import feng_gb300 as fe
from helpers import problem_spaces
from oracle.oracle import OracleProblem, ns_mms_source, taylor_hood

from conftest import load_golden


def _xy(g):
    return np.stack([g["x"], g["y"]], 1)[g["tri"]]


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name", ["kovasznay_th_8", "ns_mms_th_8"])
def test_generic_forms_match_reference_on_triangles(name):
    g = load_golden(name)
    kov = name.startswith("kovasznay")
    mu = 1.0 / float(g["re"]) if kov else 1.0
    vals, rhs = taylor_hood(g["adr"], _xy(g), g["quad"], g["u0"], int(g["nInc"]), g["ia"], g["ja"],
                            conv=-1.0, sigma=1.0, mu=mu, divu=1.0, source=None if kov else ns_mms_source)
    assert _rel(vals, g["values0"]) <= 1e-12
    assert _rel(rhs, g["rhs0"]) <= 1e-12


def test_generic_forms_match_c_oracle_with_mass_and_source():
    """Transient mass (with c0 and udot) and a constant vector source, the
    terms the steady fixtures do not hold, against the C oracle."""
    g = load_golden("kovasznay_th_8")
    mesh = fe.Mesh2DP1.generate_square(8, -0.5, 1.5, -0.5, 1.5, jitter=0.1, seed=1)
    num, _ = problem_spaces("ns_kovasznay", mesh)
    forms = [fe.feSysElm_TransientVectorMass(0.7), fe.feSysElm_VectorConvectiveAcceleration(1.0),
             fe.feSysElm_MixedDivergence(1.0), fe.feSysElm_DivergenceNewtonianStress(-1.0, 0.05),
             fe.feSysElm_VectorSource(fe.api.SRC_CONST_VEC, (0.3, -0.7))]
    rng = np.random.default_rng(4)
    u, udot = g["u0"], rng.uniform(-1, 1, len(g["u0"]))
    c0 = 150.0
    n_inc, quad = int(g["nInc"]), g["quad"]
    op = OracleProblem(num.elem_type, g["adr"], _xy(g).reshape(-1, 6), n_inc, int(g["nDofs"]),
                       g["color_offsets"], g["color_elements"], g["ia"], g["ja"], (quad[:, 0], quad[:, 1], quad[:, 2]),
                       forms)
    vals, rhs = taylor_hood(g["adr"], _xy(g), quad, u, n_inc, g["ia"], g["ja"], conv=1.0, sigma=-1.0, mu=0.05,
                            divu=1.0, mass=0.7, udot=udot, c0=c0,
                            source=lambda x, y: (np.full_like(x, 0.3), np.full_like(x, -0.7)))
    assert _rel(vals, op.matrix(u, c0)) <= 1e-12
    assert _rel(rhs, op.residual(u, udot)) <= 1e-12


def _tet_case(n=2, seed=5):
    mesh = fe.Mesh3DP1.generate_cube(n, jitter=0.05, seed=seed)
    u = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 4)
    uB = fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 4)
    p = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "Domaine", 4)
    num = fe.feMetaNumber(mesh, [u, uB, p], [uB])
    st = num.setup()
    a = mesh.arrays()
    xyz = np.stack([a["x"], a["y"], a["z"]], 1)[a["tet"]]
    quad = load_golden("diffusion3d_p2_4")["quad"]  # the reference's degree-4 tetrahedral rule
    ia, ja = st.pattern()
    return st, xyz, quad, ia, ja


def test_tet_forms_jacobian_is_the_residual_derivative():
    st, xyz, quad, ia, ja = _tet_case()
    assert st.nloc == 34
    rng = np.random.default_rng(2)
    u = rng.uniform(-1, 1, st.nDofs)
    udot = rng.uniform(-1, 1, st.nDofs)
    kw = dict(conv=1.0, sigma=-1.0, mu=0.1, divu=1.0, mass=1.0, udot=udot, c0=0.0,
              source=lambda x, y, z: (np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z), 0 * x, 0 * x))
    adr = st.elementDofs()
    vals, _ = taylor_hood(adr, xyz, quad, u, st.nInc, ia, ja, **kw)
    import scipy.sparse as sp
    A = sp.csr_matrix((vals, ja, ia), shape=(st.nInc, st.nInc))
    d = np.zeros(st.nDofs)
    d[:st.nInc] = rng.uniform(-1, 1, st.nInc)
    eps = 1e-6
    rp = taylor_hood(adr, xyz, quad, u + eps * d, st.nInc, ia, ja, **kw)[1]
    rm = taylor_hood(adr, xyz, quad, u - eps * d, st.nInc, ia, ja, **kw)[1]
    fd = -(rp - rm) / (2 * eps)   # A = -d(rhs)/du
    assert np.max(np.abs(A @ d[:st.nInc] - fd)) <= 1e-7 * np.max(np.abs(fd))


def test_tet_divergence_block_is_transposed_pressure_gradient():
    st, xyz, quad, ia, ja = _tet_case()
    rng = np.random.default_rng(3)
    u = rng.uniform(-1, 1, st.nDofs)
    vals, _ = taylor_hood(st.elementDofs(), xyz, quad, u, st.nInc, ia, ja, sigma=2.0, mu=1.0, divu=1.0)
    import scipy.sparse as sp
    A = sp.csr_matrix((vals, ja, ia), shape=(st.nInc, st.nInc)).toarray()
    x, y, fld, comp, _ = st.dofInfo()
    vel, pre = np.flatnonzero(fld[:st.nInc] == 0), np.flatnonzero(fld[:st.nInc] == 1)
    B = A[np.ix_(pre, vel)]                 # divergence rows
    Bt = A[np.ix_(vel, pre)]                # pressure-gradient columns of the stress form
    np.testing.assert_allclose(Bt, 2.0 * B.T, rtol=0, atol=1e-13 * np.max(np.abs(B)))
    K = A[np.ix_(vel, vel)]                 # viscous block: symmetric
    np.testing.assert_allclose(K, K.T, rtol=0, atol=1e-13 * np.max(np.abs(K)))
