"""CPU Newton solves of the benchmark problems, built from the oracle alone.
TEST INFRASTRUCTURE ONLY: the CPU baseline and the reference arm of bench.py
time these solves; no part of the product (the CUDA library, its host
set-up, its Python package) is imported or loaded.

A solve restates solveNewtonRaphson (src/feNonLinearSolver.cpp:38-181) with
the relative stop ||R||inf <= rel ||R0||inf: FP64 residual and Jacobian
assembly (fe_oracle.c, the reference's element kernels and colored scatter),
then a Krylov solve of J du = -R to the reference's linear tolerance 1e-8
(feLinearSystem::_rel_tol): FGMRES(50) with the saddle-point multigrid
preconditioner (fe_oracle_mg.c) for Navier-Stokes, or CG with ILU(0) for
diffusion (the configurations' CPU-runnable case), all loops on OpenMP host
threads.  Set-up (mesh, numbering, pattern, coloring, preconditioner
operators) comes from setup_oracle and is not timed.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import time
from pathlib import Path

import numpy as np

from setup_oracle import Setup, binding

_b = binding()
Forms, KStats, Problem, _p, load = _b.Forms, _b.KStats, _b.Problem, _b._p, _b.load

HERE = Path(__file__).resolve().parent
GOLDEN = HERE.parent / "tests" / "golden"

KOVASZNAY_DOMAIN = (-0.5, 1.5, -0.5, 1.5)


def reference_rule(degree: int):
    """The reference's own triangle rule of this degree (r, s, w), as its
    library reported it into the golden fixtures (degree 4: the P2
    diffusion cases; degree 8: the Navier-Stokes cases)."""
    name = {4: "diffusion_p2_8", 8: "kovasznay_th_8"}[degree]
    with np.load(GOLDEN / f"{name}.npz") as z:
        q = z["quad"]
    return q[:, 0].copy(), q[:, 1].copy(), q[:, 2].copy()


def kovasznay_fields(re: float, x, y):
    """Kovasznay (1948): u, v, p with lambda = Re/2 - sqrt(Re^2/4 + 4 pi^2)."""
    lam = re / 2.0 - math.sqrt(re * re / 4.0 + 4.0 * math.pi * math.pi)
    e = np.exp(lam * x)
    return (1.0 - e * np.cos(2 * np.pi * y), lam / (2 * np.pi) * e * np.sin(2 * np.pi * y),
            0.5 * (1.0 - np.exp(2 * lam * x)))


def _p2_ref_stiffness():
    """K[r][s][a][b] = int dphi_a/dr dphi_b/ds over the reference triangle
    (edge-midpoint rule, exact for the degree-2 integrands)."""
    pts = [(0.5, 0.0), (0.5, 0.5), (0.0, 0.5)]
    K = np.zeros((2, 2, 6, 6))
    for r, s in pts:
        l0 = 1 - r - s
        dr = np.array([-(4 * l0 - 1), 4 * r - 1, 0, 4 * (l0 - r), 4 * s, -4 * s])
        ds = np.array([-(4 * l0 - 1), 0, 4 * s - 1, -4 * r, 4 * r, 4 * (l0 - s)])
        d = (dr, ds)
        for a in range(2):
            for b in range(2):
                K[a, b] += np.outer(d[a], d[b]) / 6.0
    return K


class Problem2D:
    """A benchmark problem on the oracle set-up: the C problem descriptor,
    the essential values and the multigrid operators."""

    def __init__(self, problem: str, n: int, re: float = 40.0, seed: int = 1, jitter: float = 0.1):
        from scipy import sparse
        self.lib = load()
        dom = KOVASZNAY_DOMAIN if problem == "ns_kovasznay" else (0.0, 1.0, 0.0, 1.0)
        S = Setup("diffusion" if problem == "diffusion" else "ns", n, *dom, jitter=jitter, seed=seed)
        self.S, self.problem, self.re = S, problem, re
        th = S.elem_type == 2
        rule = reference_rule(8 if th else 4)
        f = Forms()
        f.elem_type = S.elem_type
        if th:
            f.has_conv, f.conv = 1, -1.0
            f.has_sigma, f.sigma, f.mu = 1, 1.0, 1.0 / re
            f.has_divu, f.divu = 1, 1.0
        else:
            f.has_diff, f.diff = 1, 1.0
            f.src_kind, f.src_coeff = 1, 1.0
            f.src_param[0] = -2 * np.pi ** 2
        self.keep = dict(adr=S.adr.ravel(), xy=np.ascontiguousarray(S.elem_xy).ravel(), off=S.color_offsets,
                         el=S.color_elements, ia=S.ia, ja=S.ja, qr=rule[0], qs=rule[1], qw=rule[2])
        k = self.keep
        nloc = 15 if th else 6
        self.n_inc, self.n_dofs, self.nnz = S.n_inc, S.n_dofs, len(S.ja)
        self.n_elm = len(S.tri)
        self.p = Problem(S.elem_type, self.n_elm, nloc, self.n_inc, self.n_dofs, _p(k["adr"]), _p(k["xy"]),
                         len(k["off"]) - 1, _p(k["off"]), _p(k["el"]), _p(k["ia"]), _p(k["ja"]),
                         len(k["qw"]), _p(k["qr"]), _p(k["qs"]), _p(k["qw"]), f)
        # essential values, nodewise at the DOF positions
        x, y, fld, comp = S.dof_positions()
        self.u_bc = np.zeros(self.n_dofs)
        ess = np.arange(self.n_inc, self.n_dofs)
        if th:
            u, v, pp = kovasznay_fields(re, x[ess], y[ess])
            self.u_bc[ess] = np.where(fld[ess] == 1, pp, np.where(comp[ess] == 0, u, v))
        else:
            self.u_bc[ess] = np.sin(np.pi * x[ess]) * np.sin(np.pi * y[ess])
        # multigrid operators: the scalar P2 stiffness on the velocity nodes
        # (first-component unknowns), the node -> row maps, the pressure rows
        # and their lumped P1 masses
        adr = S.adr
        vx = adr[:, 0:12:2] if th else adr
        xy = S.elem_xy
        jac = (xy[:, 2] - xy[:, 0]) * (xy[:, 5] - xy[:, 1]) - (xy[:, 3] - xy[:, 1]) * (xy[:, 4] - xy[:, 0])
        G = np.empty((len(adr), 2, 2))
        G[:, 0, 0] = (xy[:, 5] - xy[:, 1]) / jac
        G[:, 0, 1] = -(xy[:, 4] - xy[:, 0]) / jac
        G[:, 1, 0] = -(xy[:, 3] - xy[:, 1]) / jac
        G[:, 1, 1] = (xy[:, 2] - xy[:, 0]) / jac
        GG = np.einsum("erk,esk->ers", G, G)
        Ke = np.abs(jac)[:, None, None] * np.einsum("ers,rsab->eab", GG, _p2_ref_stiffness())
        rows = np.nonzero(np.isin(np.arange(self.n_inc), np.unique(vx[vx < self.n_inc])))[0]
        node = np.full(self.n_dofs, -1, np.int64)
        node[rows] = np.arange(len(rows))
        nd = node[vx]
        ok = (nd[:, :, None] >= 0) & (nd[:, None, :] >= 0)
        ii = np.broadcast_to(nd[:, :, None], Ke.shape)[ok]
        jj = np.broadcast_to(nd[:, None, :], Ke.shape)[ok]
        K = sparse.csr_matrix((Ke[ok], (ii, jj)), shape=(len(rows), len(rows)))
        K.sum_duplicates()
        K.sort_indices()
        self.K = (np.ascontiguousarray(K.indptr, np.int64), np.ascontiguousarray(K.indices, np.int32),
                  np.ascontiguousarray(K.data, np.float64))
        self.dofx = rows.astype(np.int32)
        if th:
            self.dofy = (rows + 1).astype(np.int32)   # velocity unknowns are numbered x then y per node
            pr = adr[:, 12:15]
            pm = np.zeros(self.n_dofs)
            np.add.at(pm, pr.ravel(), np.repeat(np.abs(jac) / 6.0, 3))
            self.prows = np.nonzero(np.isin(np.arange(self.n_inc), np.unique(pr[pr < self.n_inc])))[0].astype(np.int32)
            self.pmass = pm[self.prows].copy()
            if not np.array_equal(np.sort(np.concatenate([self.dofx, self.dofy, self.prows])),
                                  np.arange(self.n_inc)):
                raise RuntimeError("velocity and pressure rows do not partition the unknowns")
        else:
            self.dofy = None
            self.prows, self.pmass = np.zeros(0, np.int32), np.zeros(0)

    def residual(self, u, nthreads):
        rhs = np.zeros(self.n_inc)
        self.lib.fo_assemble_residual(C.byref(self.p), _p(u), None, _p(rhs), 0, self.n_elm, nthreads)
        return rhs

    def matrix(self, u, nthreads):
        vals = np.zeros(self.nnz)
        self.lib.fo_assemble_matrix(C.byref(self.p), _p(u), 0.0, _p(vals), 0, self.n_elm, nthreads)
        return vals


def _bind(lib):
    if getattr(lib, "_newton_bound", False):
        return
    P = C.c_void_p
    lib.fo_spmg_create.restype = P
    lib.fo_spmg_create.argtypes = [C.c_int, C.c_int64, P, P, C.c_int64, P, P, P, P, P, C.c_int64, P, P,
                                   C.c_double, C.c_double]
    lib.fo_spmg_factor.argtypes = [P, P]
    lib.fo_spmg_destroy.argtypes = [P]
    lib.fo_precond_from_spmg.restype = P
    lib.fo_precond_from_spmg.argtypes = [P]
    lib.fo_set_threads.argtypes = [C.c_int]
    lib._newton_bound = True


def newton_solve(pb: Problem2D, rel: float = 1e-8, linear_rtol: float = 1e-8, restart: int = 50,
                 max_newton: int = 30, max_krylov: int = 20000, nthreads: int | None = None,
                 precond: str | None = None):
    """One Newton solve from the boundary-initialised zero state.  Returns
    (u, stats): seconds per phase, iteration counts, final relative residual.
    precond: "mg" (the saddle-point / scalar multigrid) or "ilu0"; default
    "mg" for Navier-Stokes, "ilu0" (with CG) for diffusion."""
    lib = load()
    _bind(lib)
    nt = nthreads or os.cpu_count() or 1
    lib.fo_set_threads(nt)
    th = pb.S.elem_type == 2
    precond = precond or ("mg" if th else "ilu0")
    k = pb.keep
    t_start = time.perf_counter()
    spmg = pc = None
    if precond == "mg":
        Kia, Kja, Ka = pb.K
        spmg = lib.fo_spmg_create(4 if th else 5, pb.n_inc, _p(k["ia"]), _p(k["ja"]), len(Kia) - 1, _p(Kia),
                                  _p(Kja), _p(Ka), _p(pb.dofx), _p(pb.dofy), len(pb.prows), _p(pb.prows),
                                  _p(pb.pmass), 1.0, 1.0)
        if not spmg:
            raise RuntimeError("oracle multigrid set-up failed")
        pc = lib.fo_precond_from_spmg(spmg)
    else:
        pc = lib.fo_precond_create(1, pb.n_inc, _p(k["ia"]), _p(k["ja"]), None, None, None, 1.0)
    t_setup = time.perf_counter() - t_start
    u = pb.u_bc.copy()
    st = dict(newton_iterations=0, krylov_iterations=0, residual_s=0.0, matrix_s=0.0, factor_s=0.0,
              solve_s=0.0, converged=False)
    t0 = time.perf_counter()
    try:
        r0 = None
        while True:
            ta = time.perf_counter()
            R = pb.residual(u, nt)
            st["residual_s"] += time.perf_counter() - ta
            nr = float(np.max(np.abs(R)))
            if not np.isfinite(nr):
                raise RuntimeError("non-finite residual")
            if r0 is None:
                r0 = nr
            st["final_rel_residual"] = nr / r0 if r0 > 0 else 0.0
            if r0 == 0.0 or nr <= rel * r0:
                st["converged"] = True
                break
            if st["newton_iterations"] >= max_newton:
                break
            ta = time.perf_counter()
            A = pb.matrix(u, nt)
            st["matrix_s"] += time.perf_counter() - ta
            ta = time.perf_counter()
            if lib.fo_precond_factor(pc, _p(A)) != 0:
                raise RuntimeError("oracle preconditioner: zero pivot")
            st["factor_s"] += time.perf_counter() - ta
            du = np.zeros(pb.n_inc)
            ks = KStats()
            ta = time.perf_counter()
            lib.fo_krylov_solve(1 if th else 0, restart, max_krylov, linear_rtol, 1e-300, pb.n_inc, _p(k["ia"]),
                                _p(k["ja"]), _p(A), pc, _p(R), _p(du), C.byref(ks), nt)
            st["solve_s"] += time.perf_counter() - ta
            st["krylov_iterations"] += ks.iterations
            # the reference's residual is -R: correctSolution adds the solve of J du = R
            u[:pb.n_inc] += du
            st["newton_iterations"] += 1
    finally:
        if precond == "mg":
            lib.fo_precond_destroy(pc)
            lib.fo_spmg_destroy(spmg)
        else:
            lib.fo_precond_destroy(pc)
    st["seconds"] = time.perf_counter() - t0
    st["setup_s"] = t_setup
    st["threads"] = nt
    return u, st


def one_thread_sample(pb: Problem2D, cycle: int = 50):
    """One-thread timings of the first Newton step's pieces: residual and
    Jacobian assembly, the preconditioner set-up and one FGMRES(50) restart
    cycle (seconds; a sample, not a complete solve)."""
    lib = load()
    _bind(lib)
    lib.fo_set_threads(1)
    k = pb.keep
    u = pb.u_bc.copy()
    t0 = time.perf_counter()
    R = pb.residual(u, 1)
    t1 = time.perf_counter()
    A = pb.matrix(u, 1)
    t2 = time.perf_counter()
    Kia, Kja, Ka = pb.K
    th = pb.S.elem_type == 2
    spmg = lib.fo_spmg_create(4 if th else 5, pb.n_inc, _p(k["ia"]), _p(k["ja"]), len(Kia) - 1, _p(Kia), _p(Kja),
                              _p(Ka), _p(pb.dofx), _p(pb.dofy), len(pb.prows), _p(pb.prows), _p(pb.pmass), 1.0, 1.0)
    pc = lib.fo_precond_from_spmg(spmg)
    try:
        t3 = time.perf_counter()
        lib.fo_precond_factor(pc, _p(A))
        t4 = time.perf_counter()
        du = np.zeros(pb.n_inc)
        ks = KStats()
        lib.fo_krylov_solve(1, cycle, cycle, 1e-300, 1e-300, pb.n_inc, _p(k["ia"]), _p(k["ja"]), _p(A), pc, _p(R),
                            _p(du), C.byref(ks), 1)
        t5 = time.perf_counter()
    finally:
        lib.fo_precond_destroy(pc)
        lib.fo_spmg_destroy(spmg)
        lib.fo_set_threads(os.cpu_count() or 1)
    return {"residual_s": t1 - t0, "matrix_s": t2 - t1, "multigrid_setup_s": t3 - t2, "factor_s": t4 - t3,
            "fgmres_iterations": ks.iterations, "fgmres_s": t5 - t4,
            "ms_per_fgmres_iteration": (t5 - t4) / max(ks.iterations, 1) * 1e3}
