"""The oracle against the reference's own golden convergence outputs: P2
diffusion (tests/withLinearSolver/scalarFE_diffusion.output) and Taylor-Hood
Navier-Stokes MMS (navier_stokes_MMS.output, divergence formulation) on the
reference's meshes, solved with the oracle's residual and Jacobian and a
direct sparse solve, errors by the oracle's restatement of feNorm.

The golden files print 7 significant digits (%e); as the reference's test
(compareOutputFiles), the errors must print the same."""
import os
from pathlib import Path

import numpy as np
import pytest

from helpers import convergence_case, element_xy, essential_state, poiseuille_case, reference_l2

from feng_gb300.api import quadrature_rule
from oracle.oracle import OracleProblem, l2_error, newton_direct



def printed(v):
    return f"{float(v):.6e}"


def _oracle_errors(key, i):
    g = reference_l2()
    mesh, num, forms, spaces, fcts = convergence_case(g, key, i)
    st = num.setup(256)
    ia, ja = st.pattern()
    off, el = st.coloring()
    adr, xy = st.elementDofs(), element_xy(mesh)
    quad = quadrature_rule(8)
    op = OracleProblem(num.elem_type, adr, xy, st.nInc, st.nDofs, off, el, ia, ja, quad,
                       [f.sysElm for f in forms])
    u, its = newton_direct(op, essential_state(num, fcts))
    assert its < 20
    return g, [l2_error(num.elem_type, adr, xy, u, quad, fct, field) for field, fct in enumerate(fcts)]


@pytest.mark.parametrize("i", [1, 2, 3, 4])
def test_oracle_diffusion_p2_errors_match_reference_output(i):
    g, (e,) = _oracle_errors("diff", i)
    assert printed(e) == printed(g["diff_err_u"][i - 1])


@pytest.mark.parametrize("i", [1, 2, 3, 4])
def test_oracle_navier_stokes_mms_errors_match_reference_output(i):
    g, (eu, ep) = _oracle_errors("ns", i)
    assert printed(eu) == printed(g["ns_err_u"][i - 1])
    assert printed(ep) == printed(g["ns_err_p"][i - 1])


def test_fixture_meshes_read_back_from_the_reference_files():
    """Where the reference checkout exists: the fixture arrays are what this
    package's msh reader makes of the reference's mesh files."""
    import feng_gb300 as fe
    from conftest import reference_root
    root = reference_root()
    if root is None:
        pytest.skip("reference checkout absent")
    ref = root / "data"
    g = reference_l2()
    for key, sub in (("diff", "mmsMeshes/square"), ("ns", "square")):
        for i in range(1, 5):
            a = fe.Mesh2DP1.from_msh(ref / f"{sub}{i}.msh").arrays()
            np.testing.assert_array_equal(a["x"], g[f"{key}{i}_x"])
            np.testing.assert_array_equal(a["tri"], g[f"{key}{i}_tri"])
            np.testing.assert_array_equal(a["bnd"], g[f"{key}{i}_bnd"])
    pm = ref / "poiseuille0.msh"
    a = fe.Mesh2DP1.from_msh(pm, domain="Domain", boundary=("NoSlip", "Inlet"), point=None).arrays()
    for k in ("x", "y", "tri", "bnd"):
        np.testing.assert_array_equal(a[k], g[f"pois_{k}"])
    assert a["point"] == -1
    o = fe.Mesh2DP1.from_msh(pm, domain="Domain", boundary=("Outlet",), point=None).arrays()
    np.testing.assert_array_equal(o["bnd"], g["pois_outlet"])


def _poiseuille(stokes, constrain_outlet=True):
    g = reference_l2()
    mesh, num, forms, rows, (uex, pex) = poiseuille_case(g, stokes)
    st = num.setup(256)
    ia, ja = st.pattern()
    off, el = st.coloring()
    adr, xy = st.elementDofs(), element_xy(mesh)
    quad = quadrature_rule(8)
    op = OracleProblem(num.elem_type, adr, xy, st.nInc, st.nDofs, off, el, ia, ja, quad,
                       [f.sysElm for f in forms])
    u0 = essential_state(num, [uex, lambda xx, yy: (np.zeros_like(xx),)])
    # feNLSolverOptions{1e-10, 1e-10, 1e4, 10, ...}: at most 11 iterations.
    u, its = newton_direct(op, u0, max_iter=11, rows=rows if constrain_outlet else ())
    assert its < 11
    return rows, [l2_error(num.elem_type, adr, xy, u, quad, f, field) for field, f in enumerate((uex, pex))]


@pytest.mark.parametrize("stokes", [False, True], ids=["navier_stokes", "stokes"])
def test_oracle_poiseuille_is_exact(stokes):
    """The reference's Poiseuille tests (tests/withLinearSolver/
    navier_stokes.cpp:368-380, stokes.cpp:358-375, P2-P1): the parabolic
    velocity and linear pressure lie in the discrete spaces, so the solution
    reproduces them; the reference asserts both L2 errors below 1e-13."""
    rows, (eu, ep) = _poiseuille(stokes)
    # Outlet x = 5: 4 vertices + 3 edge midpoints, the two wall corners essential.
    assert len(rows) == 5
    assert eu < 1e-13 and ep < 1e-13


def test_oracle_poiseuille_needs_the_outlet_constraint():
    """Without the vertical velocity constrained on the outlet the outlet is
    traction-free, which the Poiseuille flow is not (shear stress u_y != 0
    there): the errors are far from rounding level."""
    _, (eu, ep) = _poiseuille(False, constrain_outlet=False)
    assert eu > 1e-6 and ep > 1e-6


def test_oracle_l2_error_closed_forms():
    """The oracle's norm on known answers: a P2 field interpolating a
    quadratic is exact (error at rounding level), and with u_h = 0 the error
    of a constant c over the domain is |c| sqrt(area) (both components for
    the vector norm)."""
    import feng_gb300 as fe
    mesh = fe.Mesh2DP1.generate_square(10, -0.5, 1.5, -0.5, 1.5, jitter=0.1, seed=3)
    from helpers import problem_spaces
    num, _ = problem_spaces("ns_kovasznay", mesh)
    st = num.setup(256)
    x, y, fld, comp, _ = st.dofInfo()
    adr, xy = st.elementDofs(), element_xy(mesh)
    quad = quadrature_rule(8)
    def quad_u(xx, yy):
        return (xx * xx - 0.5 * xx * yy + 0.25, -yy * yy + xx)
    u = np.zeros(st.nDofs)
    qu = quad_u(x, y)
    for c in range(2):
        sel = (fld == 0) & (comp == c)
        u[sel] = qu[c][sel]
    assert l2_error(num.elem_type, adr, xy, u, quad, quad_u, 0) < 1e-13
    area = 4.0
    zero = np.zeros(st.nDofs)
    e = l2_error(num.elem_type, adr, xy, zero, quad, lambda xx, yy: (np.full_like(xx, 3.0), np.full_like(xx, 4.0)), 0)
    assert e == pytest.approx(5.0 * np.sqrt(area), rel=1e-13)
    ep = l2_error(num.elem_type, adr, xy, zero, quad, lambda xx, yy: (np.full_like(xx, -2.0),), 1)
    assert ep == pytest.approx(2.0 * np.sqrt(area), rel=1e-13)
