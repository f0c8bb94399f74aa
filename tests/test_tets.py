"""Tetrahedral meshes and the P2 diffusion oracle on them, against the
reference run on the same mesh (tests/golden/diffusion3d_p2_4.npz, made by
tests/golden/make_golden.py: the reference reads the generated msh file and
assembles feSysElm_Diffusion<3> + feSysElm_Source on feSpaceTetPn(2), then
solves).  Runs on the CPU."""
from collections import Counter
import os
from pathlib import Path

import numpy as np
import pytest

import feng_gb300 as fe
from feng_gb300._lib import FeError
from oracle.oracle import tet_p2_diffusion

GOLDEN = Path(__file__).resolve().parent / "golden"


def _golden():
    return np.load(GOLDEN / "diffusion3d_p2_4.npz")


def _sinsinsin_src(x, y, z):
    return -3 * np.pi ** 2 * np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z)


def test_cube_mesh_reproduces_fixture():
    g = _golden()
    a = fe.Mesh3DP1.generate_cube(int(g["n"]), jitter=float(g["jitter"]), seed=int(g["seed"])).arrays()
    for k in ("x", "y", "z", "tet", "bnd"):
        np.testing.assert_array_equal(a[k], g[k])


def test_cube_mesh_is_conforming_and_oriented():
    n = 5
    m = fe.Mesh3DP1.generate_cube(n, 0.0, 2.0, -1.0, 0.5, 0.0, 1.0, jitter=0.05, seed=7)
    a = m.arrays()
    assert m.sizes() == ((n + 1) ** 3, 6 * n ** 3, 12 * n * n)
    x = np.stack([a["x"], a["y"], a["z"]], 1)
    t = a["tet"]
    vol = np.einsum("ij,ij->i", x[t[:, 1]] - x[t[:, 0]],
                    np.cross(x[t[:, 2]] - x[t[:, 0]], x[t[:, 3]] - x[t[:, 0]])) / 6
    assert vol.min() > 0
    assert vol.sum() == pytest.approx(2.0 * 1.5 * 1.0, rel=1e-13)
    faces = Counter(tuple(sorted(tt[f])) for tt in t for f in ([0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]))
    assert set(faces.values()) <= {1, 2}
    assert {k for k, c in faces.items() if c == 1} == {tuple(sorted(b)) for b in a["bnd"]}
    b = a["bnd"]
    normal = np.cross(x[b[:, 1]] - x[b[:, 0]], x[b[:, 2]] - x[b[:, 0]])
    assert np.all(np.einsum("ij,ij->i", normal, x[b].mean(1) - np.array([1.0, -0.25, 0.5])) > 0)
    # the seed alone fixes the jitter
    np.testing.assert_array_equal(fe.Mesh3DP1.generate_cube(n, 0.0, 2.0, -1.0, 0.5, 0.0, 1.0, jitter=0.05,
                                                            seed=7).arrays()["x"], a["x"])


def test_cube_mesh_arguments():
    for kw in (dict(n=0), dict(n=2, jitter=0.3), dict(n=2, x1=-1.0)):
        with pytest.raises(FeError):
            fe.Mesh3DP1.generate_cube(**kw)


def test_reference_reads_cube_mesh_as_generated():
    """The reference's reader takes the file: 6 n^3 tetrahedra, and P2 DOFs
    on the (2n+1)^3 lattice of vertices and edge midpoints, the interior
    ones unknown."""
    g = _golden()
    n = int(g["n"])
    assert len(g["adr"]) == 10 * 6 * n ** 3
    assert int(g["nDofs"]) == (2 * n + 1) ** 3 and int(g["nInc"]) == (2 * n - 1) ** 3


def test_oracle_tet_diffusion_matches_reference():
    g = _golden()
    xyz = np.stack([g["x"], g["y"], g["z"]], 1)[g["tet"]]
    vals, rhs = tet_p2_diffusion(g["adr"], xyz, g["quad"], g["u0"], int(g["nInc"]), g["ia"], g["ja"],
                                 source=_sinsinsin_src)
    assert np.max(np.abs(vals - g["values0"])) <= 1e-12 * np.max(np.abs(g["values0"]))
    assert np.max(np.abs(rhs - g["rhs0"])) <= 1e-12 * np.max(np.abs(g["rhs0"]))


def test_oracle_tet_diffusion_solution_matches_reference():
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    g = _golden()
    n_inc = int(g["nInc"])
    xyz = np.stack([g["x"], g["y"], g["z"]], 1)[g["tet"]]
    u = g["usol"].copy()
    u[:n_inc] = 0.0
    vals, rhs = tet_p2_diffusion(g["adr"], xyz, g["quad"], u, n_inc, g["ia"], g["ja"], source=_sinsinsin_src)
    du = spl.spsolve(sp.csr_matrix((vals, g["ja"], g["ia"]), shape=(n_inc, n_inc)).tocsc(), rhs)
    u[:n_inc] += du
    assert np.max(np.abs(u - g["usol"])) <= 1e-8 * np.max(np.abs(g["usol"]))
    # The vertex values approximate u = sin(pi x) sin(pi y) sin(pi z).
    adr = g["adr"].reshape(-1, 10)
    v, d = g["tet"].reshape(-1), adr[:, :4].reshape(-1)
    exact = np.sin(np.pi * g["x"][v]) * np.sin(np.pi * g["y"][v]) * np.sin(np.pi * g["z"][v])
    assert np.max(np.abs(u[d] - exact)) < 0.02


def _tet_numbering(mesh):
    uB = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 2, "U", "Bord", 4)
    u = fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 2, "U", "Domaine", 4)
    return fe.feMetaNumber(mesh, [uB, u], [uB])


def test_tet_setup_bit_exact():
    """Numbering, element DOF tables, coloring and CSR pattern built here on
    the generated mesh equal the reference's on the same msh file."""
    g = _golden()
    mesh = fe.Mesh3DP1.generate_cube(int(g["n"]), jitter=float(g["jitter"]), seed=int(g["seed"]))
    num = _tet_numbering(mesh)
    assert num.elem_type == fe.api.ELEM_TET_P2
    st = num.setup()
    assert (st.nInc, st.nDofs, st.nloc) == (int(g["nInc"]), int(g["nDofs"]), 10)
    np.testing.assert_array_equal(st.elementDofs().reshape(-1), g["adr"])
    ia, ja = st.pattern()
    np.testing.assert_array_equal(ia, g["ia"])
    np.testing.assert_array_equal(ja, g["ja"])
    off, el = st.coloring()
    np.testing.assert_array_equal(off, g["color_offsets"])
    np.testing.assert_array_equal(el, g["color_elements"])
    # DOF locations: vertices and edge midpoints
    x, y, f, c, isv = st.dofInfo()
    z = st.dofZ()
    adr = g["adr"].reshape(-1, 10)
    xyz = np.stack([g["x"], g["y"], g["z"]], 1)
    np.testing.assert_array_equal(np.stack([x, y, z], 1)[adr[:, :4]], xyz[g["tet"]])
    assert np.all(isv[adr[:, :4]] == 1) and np.all(isv[adr[:, 4:]] == 0)


def test_tet_setup_is_deterministic():
    """The set-up of a larger mesh (threaded pattern build) is the same twice."""
    m = fe.Mesh3DP1.generate_cube(10, jitter=0.05, seed=3)
    a = _tet_numbering(m).setup()
    b = _tet_numbering(m).setup()
    np.testing.assert_array_equal(a.pattern()[1], b.pattern()[1])
    np.testing.assert_array_equal(a.elementDofs(), b.elementDofs())


def _cube(g, i):
    return fe.Mesh3DP1.from_arrays(*(g[f"cube{i}_{k}"] for k in ("x", "y", "z", "tet", "bnd")))


@pytest.mark.parametrize("i", [1, 2, 3])
def test_tet_setup_on_reference_meshes_bit_exact(i):
    """The reference's own Gmsh meshes data/cube1-3.msh (read by this
    package's reader, tests/golden/norms/make_reference_norms.py): element
    DOF tables, CSR pattern and coloring equal the reference's."""
    from helpers import reference_l2
    g = reference_l2()
    st = _tet_numbering(_cube(g, i)).setup()
    np.testing.assert_array_equal(st.elementDofs().reshape(-1), g[f"cube{i}_adr"])
    ia, ja = st.pattern()
    np.testing.assert_array_equal(ia, g[f"cube{i}_ia"])
    np.testing.assert_array_equal(ja, g[f"cube{i}_ja"])
    off, el = st.coloring()
    np.testing.assert_array_equal(off, g[f"cube{i}_color_offsets"])
    np.testing.assert_array_equal(el, g[f"cube{i}_color_elements"])


def test_tet_interpolation_errors_match_reference_output():
    """tests/withoutLinearSolver/interpolationScalar.output, "Dimension 3 -
    Lagrange elements P2": x^6 + y^6 interpolated at the P2 nodes of
    data/cube1-3.msh, L2 error with the degree-12 rule, printed with 7
    significant digits (interpolation.cpp:12-100)."""
    from helpers import reference_l2
    from oracle.oracle import l2_error_tet
    g = reference_l2()
    for i in range(1, 4):
        mesh = _cube(g, i)
        st = _tet_numbering(mesh).setup()
        x, y, *_ = st.dofInfo()
        u = x ** 6 + y ** 6
        xyz = np.stack([g[f"cube{i}_x"], g[f"cube{i}_y"], g[f"cube{i}_z"]], 1)[g[f"cube{i}_tet"]]
        e = l2_error_tet(st.elementDofs(), xyz, u, g["tet_quad12"], lambda a, b, c: a ** 6 + b ** 6)
        assert len(g[f"cube{i}_tet"]) == g["interp3d_p2_nelm"][i - 1]
        assert f"{e:.6e}" == f"{float(g['interp3d_p2_err'][i - 1]):.6e}"


def test_tet_reader_reads_reference_files():
    """Where the reference checkout exists: the fixture arrays are what the
    reader makes of data/cube1-3.msh."""
    from helpers import reference_l2
    from conftest import reference_root
    root = reference_root()
    if root is None:
        pytest.skip("reference checkout absent")
    ref = root / "data"
    g = reference_l2()
    for i in range(1, 4):
        a = fe.Mesh3DP1.from_msh(ref / f"cube{i}.msh").arrays()
        for k in ("x", "y", "z", "tet", "bnd"):
            np.testing.assert_array_equal(a[k], g[f"cube{i}_{k}"])


def test_msh_readers_refuse_truncated_files(tmp_path):
    """A file cut anywhere in its node or element sections is an error, not
    a mesh read from uninitialised counts."""
    m3 = fe.Mesh3DP1.generate_cube(2, seed=1)
    m3.write_msh(tmp_path / "c.msh")
    m2 = fe.Mesh2DP1.generate_square(4)
    m2.write_msh(tmp_path / "s.msh")
    for name, reader in (("c.msh", fe.Mesh3DP1.from_msh), ("s.msh", fe.Mesh2DP1.from_msh)):
        text = (tmp_path / name).read_text()
        start = text.index("$Nodes")
        for frac in (0.1, 0.3, 0.5, 0.7, 0.9):
            cut = start + int((len(text) - start) * frac)
            (tmp_path / "t.msh").write_text(text[:cut])
            with pytest.raises(FeError):
                reader(tmp_path / "t.msh")


@pytest.mark.parametrize("deg", range(1, 9))
def test_tet_rules_are_exact_and_match_the_reference(deg):
    """Each tetrahedral rule integrates every monomial of its degree to
    rounding, and equals the reference's rule of that degree as a point set.
    The reference tabulates 13 decimals (5e-13); at degree 8 two 4-point
    orbits carry weights of 2e-4 and 2e-3, so the moments fix their
    positions only to about 2e-11."""
    import math
    from helpers import reference_l2
    r, s, t, w = fe.api.tet_quadrature_rule(deg)
    for i in range(deg + 1):
        for j in range(deg + 1 - i):
            for k in range(deg + 1 - i - j):
                exact = math.factorial(i) * math.factorial(j) * math.factorial(k) / math.factorial(i + j + k + 3)
                assert abs(np.sum(w * r ** i * s ** j * t ** k) - exact) <= 1e-16
    ref = reference_l2()[f"tet_quad{deg}"]
    mine = np.stack([r, s, t, w], 1)
    assert mine.shape == ref.shape
    order = lambda a: np.lexsort(np.round(a[:, :3], 8).T[::-1])
    assert np.max(np.abs(mine[order(mine)] - ref[order(ref)])) <= (5e-11 if deg == 8 else 1e-12)
