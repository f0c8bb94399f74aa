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


def _mms3d():
    """Divergence-free u = curl(0, 0, sin(pi x) sin(pi y) sin(pi z)),
    p = cos(pi x) cos(pi y) cos(pi z), and the source making them solve the
    forms conv +1, stress -1 (mu = 1), divergence +1:
    f = -(u.grad)u - grad p + lap u, lap u = -3 pi^2 u."""
    pi = np.pi

    def trig(x, y, z):
        return np.sin(pi * x), np.cos(pi * x), np.sin(pi * y), np.cos(pi * y), np.sin(pi * z), np.cos(pi * z)

    def u(x, y, z):
        sx, cx, sy, cy, sz, cz = trig(x, y, z)
        return (pi * sx * cy * sz, -pi * cx * sy * sz, 0 * x)

    def p(x, y, z):
        sx, cx, sy, cy, sz, cz = trig(x, y, z)
        return (cx * cy * cz,)

    def f(x, y, z):
        sx, cx, sy, cy, sz, cz = trig(x, y, z)
        uu = u(x, y, z)
        g = [[pi * pi * cx * cy * sz, pi * pi * sx * sy * sz], [-pi * pi * sx * sy * sz, -pi * pi * cx * cy * sz],
             [pi * pi * sx * cy * cz, -pi * pi * cx * sy * cz]]          # g[m][n] = d_m u_n, n < 2
        gp = (-pi * sx * cy * cz, -pi * cx * sy * cz, -pi * cx * cy * sz)
        conv = [sum(uu[m] * g[m][n] for m in range(3)) for n in range(2)] + [0 * x]
        return tuple(-conv[n] - gp[n] - 3 * pi * pi * uu[n] for n in range(3))

    return u, p, f


def _solve_mms3d(n, quad):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    from oracle.oracle import TET_EDGES, p2_basis
    uex, pex, src = _mms3d()
    mesh = fe.Mesh3DP1.generate_cube(n, jitter=0.05, seed=1)
    spaces = [fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 4),
              fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 4),
              fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "Domaine", 4),
              fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "Bord", 4)]
    st = fe.feMetaNumber(mesh, spaces, [spaces[1], spaces[3]]).setup()
    a = mesh.arrays()
    xyz = np.stack([a["x"], a["y"], a["z"]], 1)[a["tet"]]
    ia, ja = st.pattern()
    adr = st.elementDofs().reshape(-1, 34)
    x, y, fld, comp, _ = st.dofInfo()
    z = st.dofZ()
    sol = np.zeros(st.nDofs)
    ess = np.arange(st.nInc, st.nDofs)
    ue, pe = uex(x[ess], y[ess], z[ess]), pex(x[ess], y[ess], z[ess])[0]
    sol[ess] = np.where(fld[ess] == 0, np.choose(np.clip(comp[ess], 0, 2), ue), pe)
    kw = dict(conv=1.0, sigma=-1.0, mu=1.0, divu=1.0, source=src)
    for _ in range(10):
        vals, rhs = taylor_hood(adr, xyz, quad, sol, st.nInc, ia, ja, **kw)
        if np.max(np.abs(rhs)) < 1e-10:
            break
        du = spl.spsolve(sp.csr_matrix((vals, ja, ia), shape=(st.nInc, st.nInc)).tocsc(), rhs)
        sol[:st.nInc] += du
        if np.max(np.abs(du)) < 1e-12:
            break
    ref, w = quad[:, :3], quad[:, 3]
    phi, _ = p2_basis(ref, TET_EDGES)
    psi = np.concatenate([1 - ref.sum(-1, keepdims=True), ref], -1)
    det = np.linalg.det(np.stack([xyz[:, i + 1] - xyz[:, 0] for i in range(3)], -1))
    xq = np.einsum("qv,evx->eqx", psi, xyz)
    uh = np.einsum("qk,ekc->eqc", phi, sol[adr[:, :30]].reshape(-1, 10, 3))
    ph = np.einsum("qj,ej->eq", psi, sol[adr[:, 30:]])
    ux = np.stack(uex(*(xq[..., i] for i in range(3))), -1)
    px = pex(*(xq[..., i] for i in range(3)))[0]
    eu = np.sqrt(np.sum(((uh - ux) ** 2).sum(-1) * w * det[:, None]))
    ep = np.sqrt(np.sum((ph - px) ** 2 * w * det[:, None]))
    return eu, ep


def test_tet_taylor_hood_mms_converges_at_the_p2_p1_rates():
    """Navier-Stokes on tetrahedra with the oracle's forms and a direct
    Newton solve: L2 errors fall like h^3 (velocity) and h^2 (pressure)
    between the 3^3 and 6^3 meshes (measured 3.1 and 2.3)."""
    quad = load_golden("diffusion3d_p2_4")["quad"]
    (eu1, ep1), (eu2, ep2) = _solve_mms3d(3, quad), _solve_mms3d(6, quad)
    assert np.log2(eu1 / eu2) > 2.8
    assert np.log2(ep1 / ep2) > 1.9
