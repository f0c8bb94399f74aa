"""Builds tests/golden/norms/reference_l2.npz from the reference checkout:

* the meshes of two of its convergence tests, read with this package's msh
  4.1 reader and stored as arrays (vertices, triangles, boundary lines,
  pressure point):
    - data/mmsMeshes/square1-4.msh (tests/withLinearSolver/scalarFE.cpp:772)
    - data/square1-4.msh            (tests/withLinearSolver/navier_stokes.cpp:149)
* the channel mesh of the Poiseuille tests, data/poiseuille0.msh
  (tests/withLinearSolver/navier_stokes.cpp:297, stokes.cpp:286): the
  triangles of "Domain", the lines of "NoSlip" and "Inlet" (the essential
  boundary) and the lines of "Outlet";
* the tetrahedral meshes data/cube1-3.msh of the interpolation test
  (tests/withoutLinearSolver/interpolation.cpp:50), read with this package's
  reader, with the reference's own element DOF tables, CSR pattern and
  coloring for P2 spaces on them (the reference harness, oracle/ref_harness.cpp,
  diffusion3d) and its tetrahedral rules of degrees 1-8 and 12;
* the L2 errors those tests print in their golden output files:
    - tests/withLinearSolver/scalarFE_diffusion.output, block "P2 field 0"
      (P2 diffusion, u = sin(pi x) sin(pi y), quadrature degree 8)
    - tests/withLinearSolver/navier_stokes_MMS.output, "Divergence
      formulation" blocks (Taylor-Hood P2-P1 MMS, velocity and pressure)
    - tests/withoutLinearSolver/interpolationScalar.output, block
      "Dimension 3 - Lagrange elements P2" (nodal P2 interpolation of
      x^6 + y^6 on the cubes, quadrature degree 12).

Run where the reference exists:  python tests/golden/norms/make_reference_norms.py [REF_ROOT]
"""
import os
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[2]))

import feng_gb300 as fe  # noqa: E402


def parse_block(text, header):
    """(nElm, error) rows of the table that follows `header`."""
    lines = text.splitlines()
    i = lines.index(header)
    rows = []
    for ln in lines[i + 2:]:
        parts = ln.split()
        if len(parts) != 3:
            break
        rows.append((int(parts[0]), float(parts[1])))
    return np.array([r[0] for r in rows]), np.array([r[1] for r in rows])


def main(ref=Path("/root/reference")):
    out = {}
    for key, sub in (("diff", "data/mmsMeshes/square"), ("ns", "data/square")):
        for i in range(1, 5):
            m = fe.Mesh2DP1.from_msh(ref / f"{sub}{i}.msh")
            a = m.arrays()
            out[f"{key}{i}_x"], out[f"{key}{i}_y"] = a["x"], a["y"]
            out[f"{key}{i}_tri"], out[f"{key}{i}_bnd"] = a["tri"], a["bnd"]
            out[f"{key}{i}_point"] = np.int32(a["point"])
    pm = ref / "data/poiseuille0.msh"
    a = fe.Mesh2DP1.from_msh(pm, domain="Domain", boundary=("NoSlip", "Inlet"), point=None).arrays()
    out["pois_x"], out["pois_y"], out["pois_tri"], out["pois_bnd"] = a["x"], a["y"], a["tri"], a["bnd"]
    out["pois_outlet"] = fe.Mesh2DP1.from_msh(pm, domain="Domain", boundary=("Outlet",), point=None).arrays()["bnd"]
    root = HERE.parents[2]
    subprocess.run(["make", "-C", str(root / "oracle"), "ref", f"REF={ref}", "-j8"], check=True,
                   capture_output=True)
    for i in range(1, 4):
        cm = ref / f"data/cube{i}.msh"
        a = fe.Mesh3DP1.from_msh(cm).arrays()
        for k in ("x", "y", "z", "tet", "bnd"):
            out[f"cube{i}_{k}"] = a[k]
        with tempfile.TemporaryDirectory() as td:
            subprocess.run([str(root / "oracle/_ref/ref_harness"), str(cm), "diffusion3d", td, "1", "1"], check=True,
                           env={**os.environ, "FE_HARNESS_QDEG": "12"})
            td = Path(td)
            out[f"cube{i}_adr"] = np.fromfile(td / "adr.i64", np.int64)
            out[f"cube{i}_ia"] = np.fromfile(td / "ia.i64", np.int64)
            out[f"cube{i}_ja"] = np.fromfile(td / "ja.i64", np.int64)
            out[f"cube{i}_color_offsets"] = np.fromfile(td / "color_offsets.i64", np.int64)
            out[f"cube{i}_color_elements"] = np.fromfile(td / "color_elements.i32", np.int32)
            out["tet_quad12"] = np.fromfile(td / "quad.f64").reshape(-1, 4)
    # The reference's tetrahedral rules of degrees 1-8 (low degrees make the
    # harness's P2 solve singular after the rule is written: not checked).
    for deg in range(1, 9):
        with tempfile.TemporaryDirectory() as td:
            subprocess.run([str(root / "oracle/_ref/ref_harness"), str(ref / "data/cube1.msh"), "diffusion3d", td,
                            "1", "1"], env={**os.environ, "FE_HARNESS_QDEG": str(deg)}, capture_output=True)
            out[f"tet_quad{deg}"] = np.fromfile(Path(td) / "quad.f64").reshape(-1, 4)
    t = (ref / "tests/withoutLinearSolver/interpolationScalar.output").read_text()
    out["interp3d_p2_nelm"], out["interp3d_p2_err"] = parse_block(t, "Dimension 3 - Lagrange elements P2")
    t = (ref / "tests/withLinearSolver/scalarFE_diffusion.output").read_text()
    out["diff_nelm"], out["diff_err_u"] = parse_block(t, "Diffusion - Error on u - Lagrange elements P2 field 0")
    t = (ref / "tests/withLinearSolver/navier_stokes_MMS.output").read_text()
    blocks = [m.start() for m in re.finditer("Navier-Stokes MMS - Divergence formulation - Error on u", t)]
    assert len(blocks) == 1
    out["ns_nelm"], out["ns_err_u"] = parse_block(t, "Navier-Stokes MMS - Divergence formulation - Error on u")
    _, out["ns_err_p"] = parse_block(t, "Navier-Stokes MMS - Divergence formulation - Error on p")
    for key in ("diff", "ns"):
        for i in range(1, 5):
            assert len(out[f"{key}{i}_tri"]) == out[f"{key}_nelm"][i - 1]
    np.savez_compressed(HERE / "reference_l2.npz", **out)
    print({k: v for k, v in out.items() if "err" in k or "nelm" in k})


if __name__ == "__main__":
    main(*(Path(a) for a in sys.argv[1:]))
