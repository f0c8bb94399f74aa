"""Legacy VTK export (fe_export_vtk) against the files the reference's own
exporter (feExporterVTK::writeStep, src/feExporter.cpp:854-990) wrote for the
golden solutions (tests/golden/make_golden.py, keys "vtk" and "vtk_p").

Every line but the field values must be the same text: header, points (mesh
vertices, then edge midpoints in ascending vertex-pair order), cells, cell
types, field headers and field order.  Field values are the same text too,
except where the reference evaluates a P2 or P1 interpolant at a located
midpoint and this exporter writes the edge DOF (P2) or the mean of the two
vertex values (P1): those agree to rounding, so a value may print differently
only where both files hold a number at rounding level (below 1e-15 of the
field's largest magnitude).  Runs on the CPU."""
from pathlib import Path

import numpy as np
import pytest

import feng_gb300 as fe
from feng_gb300._lib import FeError

from helpers import golden_mesh, problem_spaces

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["diffusion_p2_8", "diffusion_p2_16", "kovasznay_th_8", "ns_mms_th_8", "cavity_bdf2_8"]


def _case(name):
    g = np.load(GOLDEN / f"{name}.npz")
    mesh = golden_mesh(g)
    num, _ = problem_spaces(str(g["problem"]), mesh, float(g["re"]))
    return g, mesh, num


def _fields(lines):
    """{name: (first value line, components, nodes)} of the POINT_DATA part."""
    i = next(k for k, ln in enumerate(lines) if ln.startswith("FIELD FieldData"))
    out, k = {}, i + 1
    for _ in range(int(lines[i].split()[2])):
        name, w, n, _ = lines[k].split()
        out[name] = (k + 1, int(w), int(n))
        k += 1 + int(w) * int(n)
    assert k == len(lines)
    return out


def _compare(ref_text, mine_text):
    a, b = ref_text.splitlines(), mine_text.splitlines()
    assert len(a) == len(b)
    fa, fb = _fields(a), _fields(b)
    assert list(fa.items()) == list(fb.items())  # names, order, sizes
    value_lines = set()
    for start, w, n in fa.values():
        value_lines.update(range(start, start + w * n))
    assert [x for i, x in enumerate(a) if i not in value_lines] == \
           [x for i, x in enumerate(b) if i not in value_lines]
    differing = 0
    for name, (start, w, n) in fa.items():
        va = np.array([float(x) for x in a[start:start + w * n]])
        vb = np.array([float(x) for x in b[start:start + w * n]])
        scale = np.max(np.abs(va))
        same_text = np.array(a[start:start + w * n]) == np.array(b[start:start + w * n])
        assert np.all(same_text | (np.abs(va - vb) <= 1e-15 * scale)), name
        # Only values at rounding level print differently.
        assert np.all(same_text | ((np.abs(va) <= 1e-15 * scale) & (np.abs(vb) <= 1e-15 * scale))), name
        differing += int((~same_text).sum())
    return differing


@pytest.mark.parametrize("name", CASES)
def test_vtk_matches_reference_exporter(tmp_path, name):
    g, mesh, num = _case(name)
    ex = fe.createVisualizationExporter(fe.VTK, num, g["usol"], mesh, num.spaces)
    ex.writeStep(tmp_path / "s.vtk")
    _compare(bytes(g["vtk"]).decode(), (tmp_path / "s.vtk").read_text())
    if "vtk_p" in g.files:
        ex.writeStep(tmp_path / "p.vtk", requiredFields=["P"])
        text = (tmp_path / "p.vtk").read_text()
        assert "CELL_TYPES" in text and "\n22\n" not in text  # P1 only: 3-node triangles
        assert _compare(bytes(g["vtk_p"]).decode(), text) == 0


def test_vtk_full_precision_holds_the_dofs(tmp_path):
    """With 17 digits the file holds the solution exactly: vertex and edge
    DOFs of the velocity, vertex DOFs of the pressure and their means at the
    midpoints."""
    g, mesh, num = _case("kovasznay_th_8")
    u = g["usol"]
    fe.createVisualizationExporter(fe.VTK, num, u, mesh, num.spaces).writeStep(tmp_path / "s.vtk", precision=17)
    lines = (tmp_path / "s.vtk").read_text().splitlines()
    f = _fields(lines)
    a = mesh.arrays()
    nv, ne = len(a["x"]), a["n_edges"]
    st = num.setup()
    x, y, fld, comp, isv = st.dofInfo()
    pts = np.array([[float(t) for t in ln.split()] for ln in lines[5:5 + nv + ne]])
    np.testing.assert_array_equal(pts[:nv, 0], a["x"])
    # Velocity: every DOF appears at the node of its location.
    s, w, n = f["U"]
    vel = np.array([float(t) for t in lines[s:s + w * n]]).reshape(n, 3)
    key = {(px, py): k for k, (px, py) in enumerate(map(tuple, pts[:, :2]))}
    for d in range(len(u)):
        if fld[d] == 0:
            v = u[d] if abs(u[d]) >= 1e-20 else 0.0
            assert vel[key[(x[d], y[d])], comp[d]] == v
    assert np.all(vel[:, 2] == 0)
    s, w, n = f["P"]
    p = np.array([float(t) for t in lines[s:s + n]])
    pv = np.zeros(nv)
    for d in np.flatnonzero(fld == 1):
        pv[key[(x[d], y[d])]] = u[d]
    np.testing.assert_array_equal(p[:nv], pv)
    ev = a["tri"][:, [0, 1, 1, 2, 2, 0]].reshape(-1, 2)
    te = a["tri_edges"].reshape(-1)
    ends = np.zeros((ne, 2), np.int64)
    ends[te] = ev
    order = np.lexsort((ends.max(1), ends.min(1)))
    np.testing.assert_array_equal(p[nv:], 0.5 * pv[ends[order, 0]] + 0.5 * pv[ends[order, 1]])


def test_vtk_arguments(tmp_path):
    g, mesh, num = _case("kovasznay_th_8")
    ex = fe.createVisualizationExporter(fe.VTK, num, g["usol"], mesh, num.spaces)
    ex.writeStep(tmp_path / "u.vtk", requiredFields=["U"])
    text = (tmp_path / "u.vtk").read_text()
    assert "FIELD FieldData 1\nU 3 " in text
    with pytest.raises(ValueError):
        ex.writeStep(tmp_path / "x.vtk", requiredFields=["T"])
    for prec in (-1, 18):
        with pytest.raises(FeError):
            ex.writeStep(tmp_path / "x.vtk", precision=prec)
    with pytest.raises(ValueError):
        fe.createVisualizationExporter(fe.VTK, num, g["usol"][:-1], mesh, num.spaces).writeStep(tmp_path / "x.vtk")
    with pytest.raises(FeError):
        ex.writeStep(tmp_path / "no_such_dir" / "x.vtk")
    other = fe.Mesh2DP1.generate_square(4, 0.0, 1.0, 0.0, 1.0)
    with pytest.raises(FeError, match="mesh"):
        fe.createVisualizationExporter(fe.VTK, num, g["usol"], other, num.spaces).writeStep(tmp_path / "x.vtk")
    with pytest.raises(ValueError):
        fe.createVisualizationExporter("GMSH", num, g["usol"], mesh, num.spaces)


def test_vtk_tetrahedra(tmp_path):
    """Tetrahedral export: vertices then edge midpoints, VTK_QUADRATIC_TETRA
    cells whose edge nodes sit at the midpoints of VTK's edges (0,1) (1,2)
    (0,2) (0,3) (1,3) (2,3), the DOF values at their nodes, and VTK_TETRA
    cells without mid-edge nodes when only the P1 field is written."""
    mesh = fe.Mesh3DP1.generate_cube(2, jitter=0.05, seed=4)
    spaces = [fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Domaine", 4),
              fe.createFiniteElementSpace(mesh, fe.VECTOR_LAGRANGE, 2, "U", "Bord", 4),
              fe.createFiniteElementSpace(mesh, fe.LAGRANGE, 1, "P", "Domaine", 4)]
    num = fe.feMetaNumber(mesh, spaces, [spaces[1]])
    st = num.setup()
    u = np.random.default_rng(1).uniform(-1, 1, st.nDofs)
    ex = fe.createVisualizationExporter(fe.VTK, num, u, mesh, num.spaces)
    ex.writeStep(tmp_path / "t.vtk", precision=17)
    lines = (tmp_path / "t.vtk").read_text().splitlines()
    a = mesh.arrays()
    nv, nt = len(a["x"]), len(a["tet"])
    n_nodes = int(lines[4].split()[1])
    pts = np.array([[float(v) for v in ln.split()] for ln in lines[5:5 + n_nodes]])
    np.testing.assert_array_equal(pts[:nv], np.stack([a["x"], a["y"], a["z"]], 1))
    c0 = 5 + n_nodes
    assert lines[c0] == f"CELLS {nt} {nt * 11}"
    cells = np.array([[int(v) for v in ln.split()] for ln in lines[c0 + 1:c0 + 1 + nt]])
    assert np.all(cells[:, 0] == 10)
    np.testing.assert_array_equal(cells[:, 1:5], a["tet"])
    for k, (i, j) in enumerate([(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]):
        mid = (pts[cells[:, 1 + i]] + pts[cells[:, 1 + j]]) / 2
        np.testing.assert_allclose(pts[cells[:, 5 + k]], mid, rtol=0, atol=1e-15)
    t0 = c0 + 1 + nt
    assert lines[t0] == f"CELL_TYPES {nt}" and set(lines[t0 + 1:t0 + 1 + nt]) == {"24"}
    f = _fields(lines)
    assert list(f) == ["P", "U"]
    s_, w, n = f["U"]
    vel = np.array([float(v) for v in lines[s_:s_ + w * n]]).reshape(n, 3)
    x, y, fld, comp, _ = st.dofInfo()
    z = st.dofZ()
    key = {tuple(p): i for i, p in enumerate(pts)}
    for d in np.flatnonzero(fld == 0):
        v = u[d] if abs(u[d]) >= 1e-20 else 0.0
        assert vel[key[(x[d], y[d], z[d])], comp[d]] == v
    ex.writeStep(tmp_path / "p.vtk", requiredFields=["P"])
    text = (tmp_path / "p.vtk").read_text()
    assert f"POINTS {nv} double" in text and f"CELLS {nt} {nt * 5}" in text
    assert "\n10\n" in text and "\n24\n" not in text
