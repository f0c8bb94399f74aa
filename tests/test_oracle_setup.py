"""The oracle's own set-up (oracle/setup_oracle.py: mesh, numbering, element
tables, coloring, CSR pattern) and its CPU Newton solve against the
reference library's output, at the configuration sizes too.

The CPU baseline and the reference arm of the benchmark build their systems
with this set-up, so it is pinned bit for bit: on every triangle fixture
(8 x 8 to the 64 x 64 diffusion mesh of the CPU-runnable configuration) and,
through SHA-256 digests, on the 256 x 256 Kovasznay mesh of the benchmark.
Assembly at the configuration sizes: 1e-12 relative to the max norm."""
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden_names, load_golden

sys.path.insert(0, str(ROOT / "oracle"))
import setup_oracle as so  # noqa: E402

TOL_FP64 = 1e-12


def _setup_of(g):
    dom = tuple(float(v) for v in g["domain"])
    prob = "diffusion" if str(g["problem"]) == "diffusion" else "ns"
    return so.Setup(prob, int(g["n"]), *dom, jitter=float(g["jitter"]), seed=int(g["seed"]))


def test_splitmix64_stream():
    """SplitMix64 of seed 0: the published first outputs."""
    with np.errstate(over="ignore"):
        u = so.splitmix64_uniform(0, 3)
    raw = np.array([0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F], dtype=np.uint64)
    assert np.array_equal(u, (raw >> np.uint64(11)).astype(np.float64) * (2.0 / 2 ** 53) - 1.0)


@pytest.mark.parametrize("name", golden_names() + golden_names(transient=True))
def test_oracle_setup_matches_reference(name):
    g = load_golden(name)
    S = _setup_of(g)
    assert np.array_equal(S.x, g["x"]) and np.array_equal(S.y, g["y"])
    assert np.array_equal(S.tri, g["tri"])
    assert (S.n_inc, S.n_dofs) == (int(g["nInc"]), int(g["nDofs"]))
    assert np.array_equal(S.adr.ravel(), g["adr"])
    assert np.array_equal(S.ia, g["ia"]) and np.array_equal(S.ja, g["ja"])
    assert np.array_equal(S.color_offsets, g["color_offsets"])
    assert np.array_equal(S.color_elements, g["color_elements"])


def _probe():
    with np.load(GOLDEN / "kovasznay_th_256_probe.npz") as z:
        return {k: z[k] for k in z.files}


def test_oracle_setup_matches_reference_at_256():
    """The benchmark mesh (Kovasznay 256 x 256, 588,290 unknowns, 16,984,800
    nonzeros): pattern, element tables and coloring digest-equal to the
    reference's."""
    import hashlib
    g = _probe()
    S = so.Setup("ns", int(g["n"]), *tuple(float(v) for v in g["domain"]), jitter=float(g["jitter"]),
                 seed=int(g["seed"]))
    h = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()  # noqa: E731
    assert (S.n_inc, S.n_dofs, len(S.ja)) == (int(g["nInc"]), int(g["nDofs"]), int(g["nnz"]))
    assert h(S.ia) == str(g["sha_ia"])
    assert h(S.ja.astype(np.int32)) == str(g["sha_ja"])
    assert h(S.adr.ravel()) == str(g["sha_adr"])
    assert h(S.color_offsets) == str(g["sha_color_offsets"])
    assert h(S.color_elements) == str(g["sha_color_elements"])


def test_oracle_assembly_at_256_matches_reference_probes():
    """The oracle's FP64 residual and Jacobian at the probe state against the
    reference's: residual rows and reductions, and A x_k for three seeded
    vectors, within 1e-12 relative to their max norms."""
    from newton_oracle import Problem2D
    g = _probe()
    pb = Problem2D("ns_kovasznay", int(g["n"]), float(g["re"]), seed=int(g["seed"]))
    n = pb.n_inc
    u = np.concatenate([so.splitmix64_uniform(int(g["state_seed"]), n), g["essential"]])
    assert np.allclose(pb.u_bc[n:], g["essential"], rtol=0, atol=1e-14 * np.abs(g["essential"]).max())
    rhs = pb.residual(u, 8)
    rows, w = g["rows"], so.splitmix64_uniform(int(g["w_seed"]), n)
    scale = float(g["rhs0_max"])
    assert np.max(np.abs(rhs[rows] - g["rhs0_rows"])) <= TOL_FP64 * scale
    assert abs(np.abs(rhs).max() - scale) <= TOL_FP64 * scale
    assert abs(np.linalg.norm(rhs) - float(g["rhs0_norm2"])) <= TOL_FP64 * float(g["rhs0_norm2"])
    assert abs(rhs @ w - float(g["rhs0_w"])) <= TOL_FP64 * scale * np.sqrt(n)
    vals = pb.matrix(u, 8)
    rows_of = np.repeat(np.arange(n), np.diff(pb.S.ia))
    for k, xs in enumerate(g["x_seeds"]):
        x = so.splitmix64_uniform(int(xs), n)
        ax = np.bincount(rows_of, weights=vals * x[pb.S.ja], minlength=n)
        sc = float(np.abs(g[f"ax{k}_rows"]).max())
        assert np.max(np.abs(ax[rows] - g[f"ax{k}_rows"])) <= TOL_FP64 * sc
        assert abs(np.linalg.norm(ax) - float(g[f"ax{k}_norm2"])) <= TOL_FP64 * float(g[f"ax{k}_norm2"])


def test_oracle_newton_at_64_matches_reference():
    """The CPU-runnable configuration (P2 diffusion, 64 x 64): the oracle's
    Newton solve with CG + ILU(0) against the reference's solution."""
    from newton_oracle import Problem2D, newton_solve
    g = load_golden("diffusion_p2_64")
    pb = Problem2D("diffusion", 64)
    u, st = newton_solve(pb, rel=1e-12, linear_rtol=1e-12, precond="ilu0")
    assert st["converged"]
    assert np.max(np.abs(u - g["usol"])) <= 1e-8 * np.max(np.abs(g["usol"]))


def test_oracle_saddle_point_multigrid_solves_kovasznay():
    """The oracle's saddle-point multigrid FGMRES reaches the reference's
    Kovasznay solution (8 x 8 fixture)."""
    from newton_oracle import Problem2D, newton_solve
    g = load_golden("kovasznay_th_8")
    pb = Problem2D("ns_kovasznay", 8)
    u, st = newton_solve(pb, rel=1e-12, linear_rtol=1e-12, precond="mg")
    assert st["converged"]
    assert np.max(np.abs(u - g["usol"])) <= 1e-8 * np.max(np.abs(g["usol"]))
