"""Generates the golden fixtures of the parity tests from the reference feNG
library itself.

Needs the reference checkout (default /root/reference) and a C++ compiler:
it builds oracle/_ref/ref_harness with oracle/Makefile, writes each seeded
mesh with this package's generator (the same file the backend reads), runs
the reference's spaces, numbering, coloring, CSR pattern, element kernels
and a Newton solve (or a BDF2 run of the lid-driven cavity with the
reference's BDF2Integrator; or P2 diffusion on a tetrahedral cube mesh) on it, and stores the arrays as compressed .npz
files next to this script, with the legacy VTK file the reference's exporter
(feExporterVTK::writeStep) writes for the final solution (key "vtk", the
file's bytes; "vtk_p": the pressure alone, requiredFields {"P"}).

    python tests/golden/make_golden.py [--ref /root/reference]
"""
from __future__ import annotations

import argparse
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import feng_gb300 as fe  # noqa: E402

# name, problem, n, domain, Re, seed
CASES = [
    ("diffusion_p2_8", "diffusion", 8, (0.0, 1.0, 0.0, 1.0), 40.0, 1),
    ("diffusion_p2_16", "diffusion", 16, (0.0, 1.0, 0.0, 1.0), 40.0, 2),
    ("kovasznay_th_8", "ns_kovasznay", 8, (-0.5, 1.5, -0.5, 1.5), 40.0, 1),
    ("ns_mms_th_8", "ns_mms", 8, (0.0, 1.0, 0.0, 1.0), 40.0, 3),
]
# P2 diffusion on tetrahedra (feSysElm_Diffusion<3>): name, n, seed, jitter
TETS = [
    ("diffusion3d_p2_4", 4, 1, 0.05),
]
# BDF2 lid-driven cavity from rest: name, n, Re, seed, dt, steps
TRANSIENT = [
    ("cavity_bdf2_8", 8, 100.0, 5, 0.01, 6),
]


def vtk_p(td):
    p = td / "solution_p.vtk"
    return dict(vtk_p=np.fromfile(p, np.uint8)) if p.exists() else {}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref", f"REF={args.ref}", f"-j8"],
                   check=True, capture_output=True)
    harness = ROOT / "oracle" / "_ref" / "ref_harness"
    for name, problem, n, dom, re, seed in CASES:
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            mesh = fe.Mesh2DP1.generate_square(n, *dom, jitter=0.1, seed=seed)
            mesh.write_msh(td / "mesh.msh")
            subprocess.run([str(harness), str(td / "mesh.msh"), problem, str(td), str(re), str(seed)],
                           check=True)
            meta = dict(l.split(maxsplit=1) for l in (td / "meta.txt").read_text().splitlines())
            arr = mesh.arrays()
            out = dict(
                problem=np.array(problem), n=np.int64(n), domain=np.array(dom), re=np.float64(re),
                seed=np.int64(seed), jitter=np.float64(0.1),
                nInc=np.int64(meta["nInc"]), nDofs=np.int64(meta["nDofs"]),
                quad_degree=np.int64(meta["quad_degree"]),
                x=arr["x"], y=arr["y"], tri=arr["tri"], bnd=arr["bnd"],
                ia=np.fromfile(td / "ia.i64", np.int64), ja=np.fromfile(td / "ja.i64", np.int64),
                adr=np.fromfile(td / "adr.i64", np.int64),
                color_offsets=np.fromfile(td / "color_offsets.i64", np.int64),
                color_elements=np.fromfile(td / "color_elements.i32", np.int32),
                u0=np.fromfile(td / "u0.f64"), values0=np.fromfile(td / "values0.f64"),
                rhs0=np.fromfile(td / "rhs0.f64"), usol=np.fromfile(td / "usol.f64"),
                quad=np.fromfile(td / "quad.f64").reshape(-1, 3),
                vtk=np.fromfile(td / "solution.vtk", np.uint8),
                **vtk_p(td),
            )
            np.savez_compressed(HERE / f"{name}.npz", **out)
            print(name, meta["nInc"], meta["nDofs"], len(out["ja"]))
    for name, n, seed, jitter in TETS:
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            mesh = fe.Mesh3DP1.generate_cube(n, jitter=jitter, seed=seed)
            mesh.write_msh(td / "mesh.msh")
            subprocess.run([str(harness), str(td / "mesh.msh"), "diffusion3d", str(td), "1", str(seed)], check=True)
            meta = dict(l.split(maxsplit=1) for l in (td / "meta.txt").read_text().splitlines())
            arr = mesh.arrays()
            out = dict(
                problem=np.array("diffusion3d"), n=np.int64(n), seed=np.int64(seed), jitter=np.float64(jitter),
                nInc=np.int64(meta["nInc"]), nDofs=np.int64(meta["nDofs"]),
                quad_degree=np.int64(meta["quad_degree"]),
                x=arr["x"], y=arr["y"], z=arr["z"], tet=arr["tet"], bnd=arr["bnd"],
                ia=np.fromfile(td / "ia.i64", np.int64), ja=np.fromfile(td / "ja.i64", np.int64),
                adr=np.fromfile(td / "adr.i64", np.int64),
                color_offsets=np.fromfile(td / "color_offsets.i64", np.int64),
                color_elements=np.fromfile(td / "color_elements.i32", np.int32),
                u0=np.fromfile(td / "u0.f64"), values0=np.fromfile(td / "values0.f64"),
                rhs0=np.fromfile(td / "rhs0.f64"), usol=np.fromfile(td / "usol.f64"),
                quad=np.fromfile(td / "quad.f64").reshape(-1, 4),
            )
            np.savez_compressed(HERE / f"{name}.npz", **out)
            print(name, meta["nInc"], meta["nDofs"], len(out["ja"]))
    for name, n, re, seed, dt, steps in TRANSIENT:
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            mesh = fe.Mesh2DP1.generate_square(n, 0.0, 1.0, 0.0, 1.0, jitter=0.1, seed=seed)
            mesh.write_msh(td / "mesh.msh")
            subprocess.run([str(harness), str(td / "mesh.msh"), "ns_cavity_bdf2", str(td), str(re), str(seed),
                            repr(dt), str(steps)], check=True)
            meta = dict(l.split(maxsplit=1) for l in (td / "meta.txt").read_text().splitlines())
            arr = mesh.arrays()
            out = dict(
                problem=np.array("ns_cavity_bdf2"), n=np.int64(n), domain=np.array((0.0, 1.0, 0.0, 1.0)),
                re=np.float64(re), seed=np.int64(seed), jitter=np.float64(0.1), dt=np.float64(dt),
                steps=np.int64(steps), nInc=np.int64(meta["nInc"]), nDofs=np.int64(meta["nDofs"]),
                quad_degree=np.int64(meta["quad_degree"]),
                x=arr["x"], y=arr["y"], tri=arr["tri"], bnd=arr["bnd"],
                ia=np.fromfile(td / "ia.i64", np.int64), ja=np.fromfile(td / "ja.i64", np.int64),
                adr=np.fromfile(td / "adr.i64", np.int64),
                color_offsets=np.fromfile(td / "color_offsets.i64", np.int64),
                color_elements=np.fromfile(td / "color_elements.i32", np.int32),
                usol=np.fromfile(td / "traj.f64"), quad=np.fromfile(td / "quad.f64").reshape(-1, 3),
                vtk=np.fromfile(td / "solution.vtk", np.uint8),
                **vtk_p(td),
            )
            np.savez_compressed(HERE / f"{name}.npz", **out)
            print(name, meta["nInc"], meta["nDofs"], len(out["ja"]))


if __name__ == "__main__":
    main()
