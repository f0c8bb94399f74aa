"""Generates the golden fixtures of the parity tests from the reference feNG
library itself.

Needs the reference checkout (--ref, else FENG_REFERENCE, else the location
recorded by the build in oracle/_ref/REFERENCE) and a C++ compiler:
it builds oracle/_ref/ref_harness with oracle/Makefile, writes each seeded
mesh with this package's generator (the same file the backend reads), runs
the reference's spaces, numbering, coloring, CSR pattern, element kernels
and a Newton solve (or a BDF2 run of the lid-driven cavity with the
reference's BDF2Integrator; or P2 diffusion on a tetrahedral cube mesh) on it, and stores the arrays as compressed .npz
files next to this script, with the legacy VTK file the reference's exporter
(feExporterVTK::writeStep) writes for the final solution (key "vtk", the
file's bytes; "vtk_p": the pressure alone, requiredFields {"P"}).

    python tests/golden/make_golden.py [--ref DIR] [--only NAME ...] [--c2-solution DIR]

Configuration-size cases: the 64 x 64 P2 diffusion mesh (C1) is stored in
full; the 256 x 256 Kovasznay mesh (C2, 588,290 unknowns, 17.0 M nonzeros) is
too large to store, so its fixture (kovasznay_th_256_probe) keeps SHA-256
digests of the pattern, element tables and coloring, and the residual, the
products A x_k of the assembled Jacobian with three vectors x_k and the
reference's converged solution on 8,192 seeded rows plus full-vector
reductions.  Its assembly state and the x_k are SplitMix64 draws from
seeds, so the tests redraw them.  The C2 direct solve takes about 30
minutes; --c2-solution reuses the usol.f64 of an earlier harness run on
the same mesh (the solution does not depend on the assembly state).
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
    ("diffusion_p2_64", "diffusion", 64, (0.0, 1.0, 0.0, 1.0), 40.0, 1),
]
# Probe fixtures of large cases: name, problem, n, domain, Re, mesh seed
PROBES = [
    ("kovasznay_th_256_probe", "ns_kovasznay", 256, (-0.5, 1.5, -0.5, 1.5), 40.0, 1),
]
PROBE_ROWS, PROBE_STATE_SEED, PROBE_X_SEEDS, PROBE_ROW_SEED, PROBE_W_SEED = 8192, 11, (21, 22, 23), 31, 41
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


def reference_dir(arg):
    import os
    if arg:
        return arg
    if os.environ.get("FENG_REFERENCE"):
        return os.environ["FENG_REFERENCE"]
    rec = ROOT / "oracle" / "_ref" / "REFERENCE"
    if rec.exists():
        return rec.read_text().strip()
    raise SystemExit("the reference checkout is needed: --ref DIR or FENG_REFERENCE")


def sha256(a: np.ndarray) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def probe_case(harness, name, problem, n, dom, re, seed, c2_solution):
    """Probe fixture of a large case (see the module docstring)."""
    import os
    sys.path.insert(0, str(ROOT / "oracle"))
    from setup_oracle import splitmix64_uniform
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        mesh = fe.Mesh2DP1.generate_square(n, *dom, jitter=0.1, seed=seed)
        mesh.write_msh(td / "mesh.msh")
        # the number of unknowns first (a run without state), then the state
        env = dict(os.environ, FE_HARNESS_NOSOLVE="1")
        subprocess.run([str(harness), str(td / "mesh.msh"), problem, str(td), str(re), str(seed)], check=True,
                       env=env)
        meta = dict(l.split(maxsplit=1) for l in (td / "meta.txt").read_text().splitlines())
        n_inc = int(meta["nInc"])
        splitmix64_uniform(PROBE_STATE_SEED, n_inc).tofile(td / "state.f64")
        env["FE_HARNESS_U0"] = str(td / "state.f64")
        subprocess.run([str(harness), str(td / "mesh.msh"), problem, str(td), str(re), str(seed)], check=True,
                       env=env)
        if c2_solution:
            usol = np.fromfile(Path(c2_solution) / "usol.f64")
        else:
            env.pop("FE_HARNESS_NOSOLVE")
            sol_dir = td / "solve"
            sol_dir.mkdir()
            subprocess.run([str(harness), str(td / "mesh.msh"), problem, str(sol_dir), str(re), str(seed)],
                           check=True, env=env)
            usol = np.fromfile(sol_dir / "usol.f64")
        ia = np.fromfile(td / "ia.i64", np.int64)
        ja = np.fromfile(td / "ja.i64", np.int64).astype(np.int32)
        vals = np.fromfile(td / "values0.f64")
        rhs0 = np.fromfile(td / "rhs0.f64")
        u0 = np.fromfile(td / "u0.f64")
        rows_of = np.repeat(np.arange(n_inc), np.diff(ia))
        rng = np.random.default_rng(PROBE_ROW_SEED)
        rows = np.sort(rng.choice(n_inc, PROBE_ROWS, replace=False)).astype(np.int64)
        w = splitmix64_uniform(PROBE_W_SEED, n_inc)
        out = dict(problem=np.array(problem), n=np.int64(n), domain=np.array(dom), re=np.float64(re),
                   seed=np.int64(seed), jitter=np.float64(0.1), nInc=np.int64(n_inc), nDofs=np.int64(meta["nDofs"]),
                   nnz=np.int64(len(ja)), quad_degree=np.int64(meta["quad_degree"]),
                   sha_ia=np.array(sha256(ia)), sha_ja=np.array(sha256(ja)),
                   sha_adr=np.array(sha256(np.fromfile(td / "adr.i64", np.int64))),
                   sha_color_offsets=np.array(sha256(np.fromfile(td / "color_offsets.i64", np.int64))),
                   sha_color_elements=np.array(sha256(np.fromfile(td / "color_elements.i32", np.int32))),
                   state_seed=np.int64(PROBE_STATE_SEED), x_seeds=np.array(PROBE_X_SEEDS, np.int64),
                   w_seed=np.int64(PROBE_W_SEED), rows=rows,
                   essential=u0[n_inc:], rhs0_rows=rhs0[rows], rhs0_w=np.float64(rhs0 @ w),
                   rhs0_norm2=np.float64(np.linalg.norm(rhs0)), rhs0_max=np.float64(np.abs(rhs0).max()),
                   rowmax_rows=np.maximum.reduceat(np.abs(vals), ia[:-1])[rows],
                   values_max=np.float64(np.abs(vals).max()),
                   usol_rows=usol[rows], usol_essential=usol[n_inc:], usol_w=np.float64(usol[:n_inc] @ w),
                   usol_max=np.float64(np.abs(usol).max()), quad=np.fromfile(td / "quad.f64").reshape(-1, 3))
        for k, xs in enumerate(PROBE_X_SEEDS):
            x = splitmix64_uniform(xs, n_inc)
            ax = np.bincount(rows_of, weights=vals * x[ja], minlength=n_inc)
            out[f"ax{k}_rows"] = ax[rows]
            out[f"ax{k}_w"] = np.float64(ax @ w)
            out[f"ax{k}_norm2"] = np.float64(np.linalg.norm(ax))
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, n_inc, meta["nDofs"], len(ja))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="")
    ap.add_argument("--only", nargs="*", default=None, help="fixture names to (re)generate")
    ap.add_argument("--c2-solution", default="", help="directory of an earlier harness run holding usol.f64")
    args = ap.parse_args()
    ref = reference_dir(args.ref)
    subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref", f"REF={ref}", f"-j8"],
                   check=True, capture_output=True)
    harness = ROOT / "oracle" / "_ref" / "ref_harness"
    want = (lambda nm: args.only is None or nm in args.only)
    for name, problem, n, dom, re, seed in PROBES:
        if want(name):
            probe_case(harness, name, problem, n, dom, re, seed, args.c2_solution)
    for name, problem, n, dom, re, seed in CASES:
        if not want(name):
            continue
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
        if not want(name):
            continue
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
        if not want(name):
            continue
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
                # transient assembly state after the last step (c0 != 0, u-dot != 0)
                u0=np.fromfile(td / "u0.f64"), udot0=np.fromfile(td / "udot0.f64"),
                values0=np.fromfile(td / "values0.f64"), rhs0=np.fromfile(td / "rhs0.f64"),
                c0=np.float64(np.fromfile(td / "c0t.f64")[0]), t_state=np.float64(np.fromfile(td / "c0t.f64")[1]),
                vtk=np.fromfile(td / "solution.vtk", np.uint8),
                **vtk_p(td),
            )
            np.savez_compressed(HERE / f"{name}.npz", **out)
            print(name, meta["nInc"], meta["nDofs"], len(out["ja"]))


if __name__ == "__main__":
    main()
