"""Host set-up against the reference library's own outputs (golden fixtures
made by tests/golden/make_golden.py): mesh generator determinism, DOF
numbering / element tables, coloring and CSR pattern bit-exact, quadrature
rules to rounding."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from helpers import golden_mesh, problem_spaces
from feng_gb300.api import quadrature_rule


ALL = golden_names() + golden_names(transient=True)


@pytest.mark.parametrize("name", ALL)
def test_mesh_generator_reproduces_fixture(name):
    g = load_golden(name)
    a = golden_mesh(g).arrays()
    assert np.array_equal(a["tri"], g["tri"])
    assert np.array_equal(a["bnd"], g["bnd"])
    np.testing.assert_allclose(a["x"], g["x"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(a["y"], g["y"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("name", ALL)
def test_numbering_pattern_coloring_bit_exact(name):
    g = load_golden(name)
    num, _ = problem_spaces(str(g["problem"]), golden_mesh(g), float(g["re"]))
    st = num.setup()
    assert (num.nInc, num.nDofs) == (int(g["nInc"]), int(g["nDofs"]))
    assert np.array_equal(st.elementDofs().ravel(), g["adr"])
    ia, ja = st.pattern()
    assert np.array_equal(ia, g["ia"]) and np.array_equal(ja, g["ja"])
    off, el = st.coloring()
    assert np.array_equal(off, g["color_offsets"]) and np.array_equal(el, g["color_elements"])


@pytest.mark.parametrize("name", golden_names())
def test_quadrature_matches_reference_rule(name):
    g = load_golden(name)
    r, s, w = quadrature_rule(int(g["quad_degree"]))
    np.testing.assert_allclose(np.stack([r, s, w], 1), g["quad"], rtol=0, atol=4e-16)


@pytest.mark.parametrize("deg", [1, 2, 4, 5, 8])
def test_quadrature_exactness(deg):
    from math import factorial
    r, s, w = quadrature_rule(deg)
    for i in range(deg + 1):
        for j in range(deg + 1 - i):
            exact = factorial(i) * factorial(j) / factorial(i + j + 2)
            assert abs(np.sum(w * r**i * s**j) - exact) < 1e-15


def test_coloring_is_vertex_disjoint_and_reference_sized():
    import feng_gb300 as fe
    m = fe.Mesh2DP1.generate_square(64, jitter=0.1, seed=1)
    num, _ = problem_spaces("diffusion", m)
    st = num.setup()
    off, el = st.coloring()
    tri = m.arrays()["tri"]
    assert st.nColors == 7  # as the reference finds on jittered structured meshes
    for c in range(st.nColors):
        v = tri[el[off[c]:off[c + 1]]].ravel()
        assert len(np.unique(v)) == len(v)
    assert sorted(el.tolist()) == list(range(len(tri)))


def test_true_problem_sizes():
    """DOF counts of the 2D configurations (P2: (2n+1)^2 nodes)."""
    import feng_gb300 as fe
    m = fe.Mesh2DP1.generate_square(64, jitter=0.1, seed=1)
    num, _ = problem_spaces("diffusion", m)
    assert num.nDofs == 16641
    m = fe.Mesh2DP1.generate_square(32, -0.5, 1.5, -0.5, 1.5, jitter=0.1, seed=1)
    num, _ = problem_spaces("ns_kovasznay", m)
    assert num.nDofs == 2 * 65 * 65 + 33 * 33


def test_threaded_setup_is_deterministic():
    """The set-up runs over host threads (pattern row by row, coloring,
    numbering): two builds of the same 96 x 96 Taylor-Hood problem give the
    same arrays, bit for bit, and the pattern rows are sorted, unique and hold
    their diagonal."""
    import feng_gb300 as fe
    out = []
    for _ in range(2):
        mesh = fe.Mesh2DP1.generate_square(96, -0.5, 1.5, -0.5, 1.5, jitter=0.1, seed=11)
        num, _ = problem_spaces("ns_kovasznay", mesh)
        st = num.setup(256)
        ia, ja = st.pattern()
        off, el = st.coloring()
        out.append((ia, ja, off, el, st.elementDofs()))
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)
    ia, ja = out[0][0], out[0][1]
    for r in range(0, len(ia) - 1, 997):
        row = ja[ia[r]:ia[r + 1]]
        assert np.all(np.diff(row) > 0) and r in row


def test_mesh_from_arrays_round_trip_and_errors():
    """fe_mesh_from_arrays rebuilds the same mesh (vertices, triangles,
    boundary lines, pressure point, edge numbering) from the arrays of
    another, and refuses out-of-range vertex indices and empty meshes."""
    import feng_gb300 as fe
    from feng_gb300._lib import FeError
    m = fe.Mesh2DP1.generate_square(12, 0.0, 1.0, 0.0, 1.0, jitter=0.1, seed=5)
    a = m.arrays()
    b = fe.Mesh2DP1.from_arrays(a["x"], a["y"], a["tri"], a["bnd"], a["point"]).arrays()
    for k in ("x", "y", "tri", "tri_edges", "bnd"):
        np.testing.assert_array_equal(a[k], b[k])
    assert a["point"] == b["point"] and a["n_edges"] == b["n_edges"]
    bad = a["tri"].copy()
    bad[3, 1] = len(a["x"])
    with pytest.raises(FeError):
        fe.Mesh2DP1.from_arrays(a["x"], a["y"], bad, a["bnd"], a["point"])
    with pytest.raises(FeError):
        fe.Mesh2DP1.from_arrays(a["x"], a["y"], a["tri"], a["bnd"], len(a["x"]))
    with pytest.raises(FeError):
        fe.Mesh2DP1.from_arrays(a["x"][:0], a["y"][:0], a["tri"][:0], a["bnd"][:0], -1)


def test_msh_reader_named_groups(tmp_path):
    """The reader maps a file's physical groups onto the three roles by name:
    the default names read as before, explicit names give the same mesh, an
    empty boundary list reads no lines, a missing domain group is an error
    that names it."""
    import feng_gb300 as fe
    from feng_gb300._lib import FeError
    m = fe.Mesh2DP1.generate_square(6, 0.0, 5.0, 0.0, 1.0, jitter=0.1, seed=2)
    path = tmp_path / "channel.msh"
    m.write_msh(path)
    a = fe.Mesh2DP1.from_msh(path).arrays()
    b = fe.Mesh2DP1.from_msh(path, domain="Domaine", boundary=["Bord"], point="PointPression").arrays()
    for k in ("x", "y", "tri", "tri_edges", "bnd"):
        np.testing.assert_array_equal(a[k], b[k])
    assert a["point"] == b["point"] == 0
    c = fe.Mesh2DP1.from_msh(path, domain="Domaine", boundary=(), point=None).arrays()
    assert c["bnd"].shape == (0, 2) and c["point"] == -1
    np.testing.assert_array_equal(a["tri"], c["tri"])
    with pytest.raises(FeError, match="Domain"):
        fe.Mesh2DP1.from_msh(path, domain="Domain", boundary=("Bord",), point=None)
