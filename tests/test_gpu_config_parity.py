"""Parity with the reference at the benchmark's configuration sizes, through
the C ABI.

* 256 x 256 Kovasznay (the benchmark mesh: 131,072 Taylor-Hood triangles,
  588,290 unknowns, 16,984,800 nonzeros), against the probe fixture
  kovasznay_th_256_probe made by the reference library: the CSR pattern,
  element tables and coloring bit-exact (SHA-256), the FP64 residual and the
  products A x_k of the FP64 Jacobian with three seeded vectors within 1e-12
  relative to their max norms (the FP32 Jacobian within 1e-5), on both
  creation routes; the converged solution within 1e-8 of the reference's
  direct-solve Newton solution, FP64 and mixed.
* The 64 x 64 P2 diffusion mesh of the CPU-runnable configuration is a full
  fixture (diffusion_p2_64) and runs through every parity test of
  test_gpu_parity.py.
* The transient Jacobian: TransientVectorMass with c0 != 0 and a nonzero
  u-dot, after six BDF2 steps of the lid-driven cavity (cavity_bdf2_8), the
  assembled matrix and residual against the reference's."""
import hashlib
import sys

import numpy as np
import pytest

import feng_gb300 as fe
from conftest import GOLDEN, ROOT, load_golden
from gpu_util import TablesSystem
from helpers import cavity_spaces, golden_mesh, rel_err

sys.path.insert(0, str(ROOT / "oracle"))
import setup_oracle as so  # noqa: E402

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12
TOL_FP32 = 1e-5
TOL_SOL = 1e-8


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def probe():
    with np.load(GOLDEN / "kovasznay_th_256_probe.npz") as z:
        g = {k: z[k] for k in z.files}
    n = int(g["nInc"])
    g["state"] = np.concatenate([so.splitmix64_uniform(int(g["state_seed"]), n), g["essential"]])
    g["w"] = so.splitmix64_uniform(int(g["w_seed"]), n)
    return g


@pytest.fixture(scope="module")
def kovasznay256(probe):
    from feng_gb300 import kovasznay
    _, num, forms = kovasznay.build(int(probe["n"]), float(probe["re"]))
    return num, forms


def _tables_of_oracle_setup(g):
    """The drop-in route's inputs (element DOFs, coordinates, coloring,
    pattern) from the oracle set-up, which is digest-equal to the reference's."""
    S = so.Setup("ns", int(g["n"]), *tuple(float(v) for v in g["domain"]), jitter=float(g["jitter"]),
                 seed=int(g["seed"]))
    assert _sha(S.ia) == str(g["sha_ia"]) and _sha(S.adr.ravel()) == str(g["sha_adr"])
    return dict(x=S.x, y=S.y, tri=S.tri, adr=S.adr.ravel(), color_offsets=S.color_offsets,
                color_elements=S.color_elements, ia=S.ia, ja=S.ja, nInc=S.n_inc, nDofs=S.n_dofs,
                quad_degree=g["quad_degree"])


def _system(route, precision, probe, kovasznay256, **kw):
    num, forms = kovasznay256
    opts = fe.LinearSolverOptions(precond="amg", precision=precision, max_iter=5000, **kw)
    if route == "tables":
        return TablesSystem(_tables_of_oracle_setup(probe), forms, opts)
    return fe.createLinearSystem(fe.CUDA, forms, num, opts)


def test_pattern_tables_coloring_at_256_bit_exact(probe, kovasznay256):
    sys_ = _system("standalone", "fp64", probe, kovasznay256)
    assert (sys_.nInc, sys_.nDofs, sys_.nnz) == (int(probe["nInc"]), int(probe["nDofs"]), int(probe["nnz"]))
    ia, ja = sys_.pattern()
    assert _sha(np.asarray(ia, np.int64)) == str(probe["sha_ia"])
    assert _sha(np.asarray(ja, np.int32)) == str(probe["sha_ja"])
    assert _sha(np.asarray(sys_.elementDofs(), np.int64).ravel()) == str(probe["sha_adr"])
    off, el = sys_.coloring()
    assert _sha(np.asarray(off, np.int64)) == str(probe["sha_color_offsets"])
    assert _sha(np.asarray(el, np.int32)) == str(probe["sha_color_elements"])


@pytest.mark.parametrize("route", ["standalone", "tables"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_assembly_at_256_matches_reference(route, precision, probe, kovasznay256):
    sys_ = _system(route, precision, probe, kovasznay256)
    sys_.setSolution(probe["state"])
    sys_.setToZero()
    sys_.assembleResiduals()
    sys_.assembleMatrices()
    sys_.synchronize()
    rhs = sys_.getRHS()
    rows = probe["rows"]
    scale = float(probe["rhs0_max"])
    # the residual is FP64 (plain) or double-float (mixed): FP64-class either way
    assert np.max(np.abs(rhs[rows] - probe["rhs0_rows"])) <= TOL_FP64 * scale
    assert abs(np.abs(rhs).max() - scale) <= TOL_FP64 * scale
    assert abs(np.linalg.norm(rhs) - float(probe["rhs0_norm2"])) <= TOL_FP64 * float(probe["rhs0_norm2"])
    vals = sys_.getMatrix()
    ia, ja = (np.asarray(a) for a in sys_.pattern())
    n = sys_.nInc
    rows_of = np.repeat(np.arange(n), np.diff(ia))
    tol = TOL_FP64 if precision == "fp64" else TOL_FP32
    rowmax = np.maximum.reduceat(np.abs(vals), ia[:-1])
    assert np.max(np.abs(rowmax[rows] - probe["rowmax_rows"])) <= tol * float(probe["values_max"])
    for k, xs in enumerate(probe["x_seeds"]):
        x = so.splitmix64_uniform(int(xs), n)
        ax = np.bincount(rows_of, weights=vals * x[ja], minlength=n)
        sc = float(np.abs(probe[f"ax{k}_rows"]).max())
        assert np.max(np.abs(ax[rows] - probe[f"ax{k}_rows"])) <= tol * sc
        assert abs(np.linalg.norm(ax) - float(probe[f"ax{k}_norm2"])) <= tol * float(probe[f"ax{k}_norm2"])


@pytest.mark.parametrize("route", ["standalone", "tables"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_newton_at_256_matches_reference_solution(route, precision, probe, kovasznay256):
    """Newton to a tight relative residual (the reference's direct solves end
    at ||R||inf ~ 1e-16), then the solution on the probe rows and its
    reductions against the reference's."""
    sys_ = _system(route, precision, probe, kovasznay256, rel_tol=1e-12 if precision == "fp64" else 1e-8)
    n = sys_.nInc
    # the reference's start: unknowns 0, its essential values
    sys_.setSolution(np.concatenate([np.zeros(n), probe["usol_essential"]]))
    nl = fe.feNLSolverOptions(tolResidual=0.0, tolCorrection=0.0, maxIter=30,
                              relResidual=1e-13 if precision == "fp64" else 1e-12,
                              linearRtolMin=0.0 if precision == "fp64" else 1e-6)
    st = fe.solveNewtonRaphson(sys_, None, nl)
    assert st["return"] == 0, st
    u = sys_.getSolution()
    scale = float(probe["usol_max"])
    assert np.max(np.abs(u[probe["rows"]] - probe["usol_rows"])) <= TOL_SOL * scale
    assert np.max(np.abs(u[n:] - probe["usol_essential"])) <= 1e-14 * scale
    assert abs(u[:n] @ probe["w"] - float(probe["usol_w"])) <= TOL_SOL * scale * np.sqrt(n)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_transient_jacobian_matches_reference(precision):
    """TransientVectorMass in the Jacobian (c0 c M) and the residual (u-dot
    M) at the reference's state after six BDF2 steps of the cavity."""
    g = load_golden("cavity_bdf2_8")
    assert float(g["c0"]) != 0.0 and np.max(np.abs(g["udot0"])) > 0
    num, forms = cavity_spaces(golden_mesh(g), float(g["re"]))
    sys_ = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond="ilu0", precision=precision))
    sys_.setSolution(g["u0"], g["udot0"])
    sys_.setTime(float(g["t_state"]), float(g["c0"]))
    sys_.setToZero()
    sys_.assembleResiduals()
    sys_.assembleMatrices()
    sys_.synchronize()
    assert rel_err(sys_.getRHS(), g["rhs0"]) <= TOL_FP64
    assert rel_err(sys_.getMatrix(), g["values0"]) <= (TOL_FP64 if precision == "fp64" else TOL_FP32)
