"""The CPU oracle: a ctypes binding of its C restatement (oracle/fe_oracle.c,
oracle/mlp_oracle.c) and numpy restatements of the error norms, the direct
Newton solve and the tetrahedral forms (P2 diffusion; Taylor-Hood forms on
triangles and tetrahedra).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product.  The C part is built by
``make -C oracle port`` into oracle/_ref/libfeoracle.so.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_ref" / "libfeoracle.so"


class Forms(C.Structure):
    _fields_ = [("elem_type", C.c_int), ("has_diff", C.c_int), ("diff", C.c_double),
                ("has_conv", C.c_int), ("conv", C.c_double), ("has_sigma", C.c_int),
                ("sigma", C.c_double), ("mu", C.c_double), ("has_divu", C.c_int),
                ("divu", C.c_double), ("has_mass", C.c_int), ("mass", C.c_double),
                ("src_kind", C.c_int), ("src_coeff", C.c_double), ("src_param", C.c_double * 4)]


class Problem(C.Structure):
    _fields_ = [("elem_type", C.c_int), ("n_elm", C.c_int64), ("nloc", C.c_int),
                ("n_inc", C.c_int64), ("n_dofs", C.c_int64), ("adr", C.c_void_p),
                ("elem_xy", C.c_void_p), ("n_colors", C.c_int), ("color_offsets", C.c_void_p),
                ("color_elements", C.c_void_p), ("ia", C.c_void_p), ("ja", C.c_void_p),
                ("nq", C.c_int), ("qr", C.c_void_p), ("qs", C.c_void_p), ("qw", C.c_void_p),
                ("forms", Forms)]


class KStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("rnorm0", C.c_double),
                ("rnorm", C.c_double)]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            subprocess.run(["make", "-C", str(HERE), "port"], check=True, capture_output=True)
        lib = C.CDLL(str(LIB))
        P = C.c_void_p
        lib.fo_assemble_residual.argtypes = [P, P, P, P, C.c_int64, C.c_int64, C.c_int]
        lib.fo_assemble_matrix.argtypes = [P, P, C.c_double, P, C.c_int64, C.c_int64, C.c_int]
        lib.fo_spmv.argtypes = [C.c_int64, P, P, P, P, P, C.c_int]
        lib.fo_precond_create.restype = P
        lib.fo_precond_create.argtypes = [C.c_int, C.c_int64, P, P, P, P, P, C.c_double]
        lib.fo_precond_factor.argtypes = [P, P]
        lib.fo_precond_apply.argtypes = [P, P, P]
        lib.fo_precond_destroy.argtypes = [P]
        lib.fo_krylov_solve.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                        C.c_int64, P, P, P, P, P, P, C.POINTER(KStats), C.c_int]
        lib.fo_constrain.argtypes = [C.c_int64, P, P, P, P, P, C.c_int64]
        lib.fo_periodicity.argtypes = [C.c_int64, P, P, P, P, P, P, C.c_int64]
        lib.mo_param_count.restype = C.c_int64
        lib.mo_param_count.argtypes = [C.c_int] * 4
        lib.mo_forward.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P, C.c_int64, P]
        lib.mo_loss_grad.restype = C.c_double
        lib.mo_loss_grad.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, P, C.c_int64, P]
        lib.mo_adam.argtypes = [P, P, P, P, C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_int]
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def forms_from(elem_type, sysElms):
    """Fused coefficients of a list of feSysElm descriptors (feng_gb300.api)."""
    f = Forms()
    f.elem_type = elem_type
    for s in sysElms:
        k = s.kind
        if k == 2:
            f.has_diff, f.diff = 1, f.diff + s.coeff
        elif k in (1, 3):
            f.src_kind, f.src_coeff = s.source, (s.coeff or 1.0)
            for i in range(4):
                f.src_param[i] = s.params[i]
        elif k == 6:
            f.has_conv, f.conv = 1, f.conv + s.coeff
        elif k == 7:
            f.has_sigma, f.sigma, f.mu = 1, s.coeff, s.coeff2
        elif k == 5:
            f.has_divu, f.divu = 1, f.divu + s.coeff
        elif k == 4:
            f.has_mass, f.mass = 1, f.mass + s.coeff
    return f


class OracleProblem:
    """Element tables + pattern + coloring + quadrature + forms, held for the C oracle."""

    def __init__(self, elem_type, adr, elem_xy, n_inc, n_dofs, color_offsets, color_elements,
                 ia, ja, quad, sysElms):
        self.lib = load()
        self.keep = dict(
            adr=np.ascontiguousarray(adr, np.int64).ravel(),
            xy=np.ascontiguousarray(elem_xy, np.float64).ravel(),
            off=np.ascontiguousarray(color_offsets, np.int64),
            el=np.ascontiguousarray(color_elements, np.int32),
            ia=np.ascontiguousarray(ia, np.int64), ja=np.ascontiguousarray(ja, np.int32),
            qr=np.ascontiguousarray(quad[0], np.float64), qs=np.ascontiguousarray(quad[1], np.float64),
            qw=np.ascontiguousarray(quad[2], np.float64))
        k = self.keep
        nloc = 6 if elem_type == 1 else 15
        self.n_inc, self.n_dofs, self.nnz = int(n_inc), int(n_dofs), len(k["ja"])
        self.n_elm = len(k["adr"]) // nloc
        self.p = Problem(elem_type, self.n_elm, nloc, self.n_inc, self.n_dofs, _p(k["adr"]), _p(k["xy"]),
                         len(k["off"]) - 1, _p(k["off"]), _p(k["el"]), _p(k["ia"]), _p(k["ja"]),
                         len(k["qw"]), _p(k["qr"]), _p(k["qs"]), _p(k["qw"]), forms_from(elem_type, sysElms))

    def residual(self, u, udot=None, begin=0, end=None, nthreads=None):
        rhs = np.zeros(self.n_inc)
        self.lib.fo_assemble_residual(C.byref(self.p), _p(np.ascontiguousarray(u)),
                                      _p(None if udot is None else np.ascontiguousarray(udot)), _p(rhs),
                                      begin, self.n_elm if end is None else end,
                                      nthreads or os.cpu_count())
        return rhs

    def matrix(self, u, c0=0.0, begin=0, end=None, nthreads=None):
        vals = np.zeros(self.nnz)
        self.lib.fo_assemble_matrix(C.byref(self.p), _p(np.ascontiguousarray(u)), c0, _p(vals), begin,
                                    self.n_elm if end is None else end, nthreads or os.cpu_count())
        return vals

    def solve(self, values, b, method=1, restart=50, max_iter=5000, rtol=1e-8, atol=1e-14,
              pc_kind=1, block_of_row=None, is_pressure=None, pmass=None, viscosity=1.0,
              nthreads=None):
        k = self.keep
        blk = None if block_of_row is None else np.ascontiguousarray(block_of_row, np.int32)
        isp = None if is_pressure is None else np.ascontiguousarray(is_pressure, np.int32)
        pm = None if pmass is None else np.ascontiguousarray(pmass, np.float64)
        pc = self.lib.fo_precond_create(pc_kind, self.n_inc, _p(k["ia"]), _p(k["ja"]), _p(blk), _p(isp),
                                        _p(pm), viscosity)
        try:
            vals = np.ascontiguousarray(values, np.float64)
            s = self.lib.fo_precond_factor(pc, _p(vals))
            if s != 0:
                raise RuntimeError("oracle preconditioner: zero pivot")
            x = np.zeros(self.n_inc)
            st = KStats()
            self.lib.fo_krylov_solve(method, restart, max_iter, rtol, atol, self.n_inc, _p(k["ia"]),
                                     _p(k["ja"]), _p(vals), pc, _p(np.ascontiguousarray(b)), _p(x),
                                     C.byref(st), nthreads or os.cpu_count())
            return x, dict(iterations=st.iterations, converged=bool(st.converged), rnorm0=st.rnorm0,
                           rnorm=st.rnorm)
        finally:
            self.lib.fo_precond_destroy(pc)


    def apply_ilu(self, values, r, block_of_row=None):
        """z = (LU)^-1 r with the serial (block-Jacobi) ILU(0) of values."""
        k = self.keep
        blk = None if block_of_row is None else np.ascontiguousarray(block_of_row, np.int32)
        pc = self.lib.fo_precond_create(1, self.n_inc, _p(k["ia"]), _p(k["ja"]), _p(blk), None, None, 1.0)
        try:
            vals = np.ascontiguousarray(values, np.float64)
            if self.lib.fo_precond_factor(pc, _p(vals)) != 0:
                raise RuntimeError("oracle ILU(0): zero pivot")
            z = np.zeros(self.n_inc)
            self.lib.fo_precond_apply(pc, _p(np.ascontiguousarray(r, np.float64)), _p(z))
            return z
        finally:
            self.lib.fo_precond_destroy(pc)


# ---- learned-guess MLP (oracle/mlp_oracle.c) ----------------------------------

def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def mlp_param_count(dims):
    return int(load().mo_param_count(*dims))


def mlp_forward(params, dims, x):
    """FP64 forward pass; dims = (nin, h1, h2, nout), x [n, nin] -> y [n, nout]."""
    params, x = _f64(params), _f64(x)
    y = np.zeros((x.shape[0], dims[3]))
    load().mo_forward(_p(params), *dims, _p(x), x.shape[0], _p(y))
    return y


def mlp_loss_grad(params, dims, x, t, mask=None):
    """Masked mean-squared loss and its gradient (packed like the parameters)."""
    params, x, t = _f64(params), _f64(x), _f64(t)
    mask = None if mask is None else _f64(mask)
    g = np.zeros(mlp_param_count(dims))
    loss = load().mo_loss_grad(_p(params), *dims, _p(x), _p(t), _p(mask), x.shape[0], _p(g))
    return loss, g


def mlp_adam(params, m, v, grad, lr, step, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step in place on FP64 copies; returns (params, m, v)."""
    params, m, v, grad = _f64(params).copy(), _f64(m).copy(), _f64(v).copy(), _f64(grad)
    load().mo_adam(_p(params), _p(m), _p(v), _p(grad), params.size, lr, beta1, beta2, eps, step)
    return params, m, v


# ---- essential components / periodicity (oracle/fe_oracle.c) -------------------

def constrain(ia, ja, values, rhs, rows=(), master=(), slave=()):
    """Copies of (values, rhs) after constrainEssentialComponents and
    applyPeriodicity as the MKL backend does them."""
    ia = np.ascontiguousarray(ia, np.int64)
    ja = np.ascontiguousarray(ja, np.int32)
    v = np.array(values, dtype=np.float64, copy=True)
    r = np.array(rhs, dtype=np.float64, copy=True)
    n = len(ia) - 1
    rows = np.ascontiguousarray(rows, np.int64)
    load().fo_constrain(n, _p(ia), _p(ja), _p(v), _p(r), _p(rows), len(rows))
    m = np.ascontiguousarray(master, np.int64)
    s = np.ascontiguousarray(slave, np.int64)
    load().fo_periodicity(n, _p(ia), _p(ja), _p(v), _p(r), _p(m), _p(s), len(m))
    return v, r


# ---- error norms and a direct Newton solve (convergence golden outputs) -------

def _p2_shape(r, s):
    """feSpaceTriP2 shape functions (src/feSpace_2D.cpp:536-566): vertex
    functions 0-2, then edge functions of edges (0,1), (1,2), (2,0)."""
    t = 1.0 - r - s
    return np.stack([t * (1 - 2 * r - 2 * s), r * (2 * r - 1), s * (2 * s - 1), 4 * r * t, 4 * r * s, 4 * s * t], -1)


def l2_error(elem_type, adr, elem_xy, u, quad, fct, field):
    """feNorm L2_ERROR / VECTOR_L2_ERROR with p = 2 (src/feNorm.cpp:323-391,
    1399-1443): over the elements in mesh order and the rule's nodes,
    sum |u_ex - u_h|^2 J w, u_h from the element's DOFs (scalar P2: local a;
    Taylor-Hood velocity: local 2a + c; Taylor-Hood pressure: local 12 + j),
    positions from the P1 geometry, J the element's Jacobian determinant;
    returns the square root."""
    r, s, w = (np.asarray(v, np.float64) for v in quad)
    xy = np.asarray(elem_xy, np.float64).reshape(-1, 6)
    adr = np.asarray(adr, np.int64)
    x0, y0, x1, y1, x2, y2 = xy.T
    det = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0)
    psi = np.stack([1 - r - s, r, s], -1)                       # nq x 3
    px = np.outer(x0, psi[:, 0]) + np.outer(x1, psi[:, 1]) + np.outer(x2, psi[:, 2])
    py = np.outer(y0, psi[:, 0]) + np.outer(y1, psi[:, 1]) + np.outer(y2, psi[:, 2])
    ex = fct(px, py)
    u = np.asarray(u, np.float64)
    if elem_type == 1 and field == 0:
        uh = [u[adr[:, :6]] @ _p2_shape(r, s).T]
    elif elem_type == 2 and field == 0:
        phi = _p2_shape(r, s)
        uh = [u[adr[:, c:12:2]] @ phi.T for c in range(2)]
    elif elem_type == 2 and field == 1:
        uh = [u[adr[:, 12:15]] @ psi.T]
    else:
        raise ValueError("no such field")
    e2 = sum((np.broadcast_to(ex[c], px.shape) - uh[c]) ** 2 for c in range(len(uh)))
    per_elem = (e2 * w[None, :]).sum(1) * det
    res = float(per_elem.sum())
    if res < 0 and abs(res) < 1e-14:
        res = abs(res)
    return np.sqrt(res)


def newton_direct(op, u, tol_residual=1e-10, tol_correction=1e-10, max_iter=20, rows=()):
    """Newton iterations on the oracle's residual and Jacobian with a direct
    sparse solve (scipy SuperLU), in feNG's convention: A du = rhs (rhs = sum
    of element Be), u[:nInc] += du; stops on the absolute max-norms of the
    residual or the correction (src/feNonLinearSolver.cpp:38-181).  `rows`
    are the unknowns of essential components (setEssentialComponent): their
    rows of A and rhs are constrained before the solve and the stop test
    (src/feNonLinearSolver.cpp:94, constrainEssentialComponents), so they
    keep their initial values."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    k = op.keep
    u = np.array(u, np.float64)
    for it in range(max_iter):
        rhs = op.residual(u)
        vals = None
        if len(rows):
            vals, rhs = constrain(k["ia"], k["ja"], op.matrix(u), rhs, rows=rows)
        if np.max(np.abs(rhs)) <= tol_residual:
            return u, it
        a = sp.csr_matrix((op.matrix(u) if vals is None else vals, k["ja"], k["ia"]),
                          shape=(op.n_inc, op.n_inc))
        du = spl.spsolve(a.tocsc(), rhs)
        u[:op.n_inc] += du
        if np.max(np.abs(du)) <= tol_correction:
            return u, it + 1
    return u, max_iter


# ---- P2 tetrahedra: diffusion + source (numpy restatement) ---------------------

# Local edges of a tetrahedron, in the order of its edge DOFs
# (_edgesOrder, src/feTetrahedron.h:31; getTetLagrangeBarycentricCoord,
# src/feTetrahedron.cpp:170-194).
TET_EDGES = ((0, 2), (2, 1), (1, 0), (1, 3), (3, 0), (3, 2))


def tet_p2_basis(r, s, t):
    """feSpaceTetPn with n = 2 (src/feSpace_3D.cpp:104-235): barycentric
    l = (1 - r - s - t, r, s, t); vertex functions l_i (2 l_i - 1), then edge
    functions 4 l_a l_b over TET_EDGES.  Returns phi (nq, 10) and the
    reference gradients d phi / d(r, s, t) (nq, 10, 3)."""
    r, s, t = (np.asarray(v, np.float64) for v in (r, s, t))
    lam = np.stack([1 - r - s - t, r, s, t], -1)
    dlam = np.array([[-1, -1, -1], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float64)
    phi = [lam[..., i] * (2 * lam[..., i] - 1) for i in range(4)]
    phi += [4 * lam[..., a] * lam[..., b] for a, b in TET_EDGES]
    dphi = [np.multiply.outer(4 * lam[..., i] - 1, dlam[i]) for i in range(4)]
    dphi += [4 * (np.multiply.outer(lam[..., b], dlam[a]) + np.multiply.outer(lam[..., a], dlam[b]))
             for a, b in TET_EDGES]
    return np.stack(phi, -1), np.stack(dphi, -2)


def tet_p2_diffusion(adr, tet_xyz, quad, u, n_inc, ia, ja, coeff=1.0, source=None):
    """CSR values and residual of feSysElm_Diffusion<3> (+ feSysElm_Source)
    on P2 tetrahedra, scattered as the MKL backend does (rows and columns of
    essential DOFs dropped; feLinearSystemMklPardiso.cpp:501-749):

      Ae_ij = sum_q k grad phi_i . grad phi_j J w       (src/feSysElm.cpp:531-556)
      Be_i  = - sum_q k grad phi_i . grad u_h J w       (src/feSysElm.cpp:558-583)
              - sum_q phi_i f(x_q) J w                  (src/feSysElm.cpp:16-27)

    with the affine map of the P1 tetrahedron (J = det [x1-x0, x2-x0, x3-x0],
    grad phi = J^-T d phi/d(r,s,t)) and x_q interpolated from the vertices.
    adr (nElm, 10); tet_xyz (nElm, 4, 3); quad (nq, 4) rows r, s, t, w;
    source(x, y, z) -> f or None."""
    adr = np.asarray(adr, np.int64).reshape(-1, 10)
    X = np.asarray(tet_xyz, np.float64).reshape(-1, 4, 3)
    q = np.asarray(quad, np.float64).reshape(-1, 4)
    jm = np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]], -1)
    det, inv = np.linalg.det(jm), np.linalg.inv(jm)
    phi, dphi = tet_p2_basis(q[:, 0], q[:, 1], q[:, 2])
    w = q[:, 3]
    grad = np.einsum("qfk,ekx->eqfx", dphi, inv)
    ae = coeff * np.einsum("eqix,eqjx,q,e->eij", grad, grad, w, det)
    gu = np.einsum("eqfx,ef->eqx", grad, np.asarray(u, np.float64)[adr])
    be = -coeff * np.einsum("eqix,eqx,q,e->ei", grad, gu, w, det)
    if source is not None:
        psi = np.stack([1 - q[:, 0] - q[:, 1] - q[:, 2], q[:, 0], q[:, 1], q[:, 2]], -1)
        xq = np.einsum("qv,evx->eqx", psi, X)
        f = source(xq[..., 0], xq[..., 1], xq[..., 2])
        be -= np.einsum("qi,eq,q,e->ei", phi, f, w, det)
    return _scatter(adr, ae, be, n_inc, ia, ja)


def _scatter(adr, ae, be, n_inc, ia, ja, mask=None):
    """MKL-style scatter of element matrices ae (nElm, nloc, nloc) and
    vectors be (nElm, nloc): entries with an essential row or column are
    dropped; mask (nloc, nloc) selects the coupled local pairs."""
    ia, ja = np.asarray(ia, np.int64), np.asarray(ja, np.int64)
    rhs = np.zeros(n_inc)
    keep = adr < n_inc
    np.add.at(rhs, adr[keep], be[keep])
    rows = np.broadcast_to(adr[:, :, None], ae.shape)
    cols = np.broadcast_to(adr[:, None, :], ae.shape)
    m = (rows < n_inc) & (cols < n_inc)
    if mask is not None:
        m &= np.asarray(mask, bool)[None]
    # Position of (r, c) in the pattern: rows in order, columns ascending
    # within a row, so row * (n + 1) + column ascends over the whole array.
    lin = np.repeat(np.arange(n_inc), np.diff(ia)) * (n_inc + 1) + ja
    want = rows[m] * (n_inc + 1) + cols[m]
    pos = np.minimum(np.searchsorted(lin, want), len(lin) - 1)
    if not np.array_equal(lin[pos], want):
        raise ValueError("an element coupling lies outside the CSR pattern")
    values = np.zeros(len(ja))
    np.add.at(values, pos, ae[m])
    return values, rhs


# ---- Taylor-Hood forms on triangles and tetrahedra (numpy restatement) ---------

TRI_EDGES = ((0, 1), (1, 2), (2, 0))


def p2_basis(ref, edges):
    """P2 Lagrange basis on a simplex of dimension d = ref.shape[-1] at the
    reference points ref (nq, d): barycentric l = (1 - sum, ref...), vertex
    functions l_i (2 l_i - 1), then 4 l_a l_b over `edges`.  Returns phi
    (nq, n) and d phi / d ref (nq, n, d)."""
    ref = np.asarray(ref, np.float64)
    d = ref.shape[-1]
    lam = np.concatenate([1 - ref.sum(-1, keepdims=True), ref], -1)
    dlam = np.vstack([-np.ones(d), np.eye(d)])
    phi = [lam[:, i] * (2 * lam[:, i] - 1) for i in range(d + 1)]
    phi += [4 * lam[:, a] * lam[:, b] for a, b in edges]
    dphi = [np.multiply.outer(4 * lam[:, i] - 1, dlam[i]) for i in range(d + 1)]
    dphi += [4 * (np.multiply.outer(lam[:, b], dlam[a]) + np.multiply.outer(lam[:, a], dlam[b])) for a, b in edges]
    return np.stack(phi, -1), np.stack(dphi, -2)


def taylor_hood(adr, vert_xyz, quad, u, n_inc, ia, ja, conv=0.0, sigma=0.0, mu=1.0, divu=0.0, mass=0.0,
                udot=None, c0=0.0, source=None):
    """CSR values and residual of the Taylor-Hood forms on triangles (d = 2,
    the reference's forms) or tetrahedra (d = 3, the same weak forms, which
    the reference does not instantiate), scattered as the MKL backend does.
    Local layout: velocity node k (vertices, then edges) component c at
    d k + c, pressure vertex j after the velocity.  Gradient convention
    (grad u)_mn = d_m u_n.  With W = J w at each quadrature node:

    VectorConvectiveAcceleration (src/feVectorSysElm.cpp:1171-1240)
      Be_kc -= conv W phi_k (u . grad u)_c
      A_kc,la += conv W phi_k (phi_l d_a u_c + delta_ca u . grad phi_l)
    DivergenceNewtonianStress (src/feVectorSysElm.cpp:1454-1530)
      Be_kc -= sigma W (p d_c phi_k - mu sum_m (d_m u_c + d_c u_m) d_m phi_k)
      A_kc,la += -sigma mu W (delta_ca grad phi_k . grad phi_l + d_a phi_k d_c phi_l)
      A_kc,pj += sigma W psi_j d_c phi_k
    MixedDivergence (src/feVectorSysElm.cpp:685-747)
      Be_pj -= divu W (div u) psi_j;  A_pj,la += divu W psi_j d_a phi_l
    TransientVectorMass (src/feVectorSysElm.cpp:390-427)
      Be_kc -= mass W udot_c phi_k;  A_kc,lc += mass c0 W phi_k phi_l
    VectorSource (src/feVectorSysElm.cpp:112-130)
      Be_kc -= W f_c(x_q) phi_k, source(*coords) -> tuple of d arrays.

    vert_xyz (nElm, d+1, d); quad (nq, d+1) rows (reference point, w)."""
    q = np.asarray(quad, np.float64)
    d = q.shape[1] - 1
    nv, edges = d + 1, (TRI_EDGES if d == 2 else TET_EDGES)
    n2 = nv + len(edges)
    nloc = d * n2 + nv
    adr = np.asarray(adr, np.int64).reshape(-1, nloc)
    X = np.asarray(vert_xyz, np.float64).reshape(-1, nv, d)
    ref, w = q[:, :d], q[:, d]
    jm = np.stack([X[:, i + 1] - X[:, 0] for i in range(d)], -1)
    det, inv = np.linalg.det(jm), np.linalg.inv(jm)
    phi, dphi = p2_basis(ref, edges)
    psi = np.concatenate([1 - ref.sum(-1, keepdims=True), ref], -1)
    G = np.einsum("qkr,erx->eqkx", dphi, inv)                 # grad phi_k
    W = det[:, None] * w[None, :]                             # (ne, nq)
    ue = np.asarray(u, np.float64)[adr]
    U, P = ue[:, :d * n2].reshape(-1, n2, d), ue[:, d * n2:]
    uq = np.einsum("qk,ekn->eqn", phi, U)
    gu = np.einsum("eqkm,ekn->eqmn", G, U)
    pq = np.einsum("qj,ej->eq", psi, P)
    ne_ = len(adr)
    bu = np.zeros((ne_, n2, d))
    bp = np.zeros((ne_, nv))
    A = np.zeros((ne_, n2, d, n2, d))
    Aup = np.zeros((ne_, n2, d, nv))
    Apu = np.zeros((ne_, nv, n2, d))
    eye = np.eye(d)
    if conv:
        ugu = np.einsum("eqm,eqmn->eqn", uq, gu)
        bu -= conv * np.einsum("eq,qk,eqc->ekc", W, phi, ugu)
        A += conv * np.einsum("zq,qk,ql,zqac->zkcla", W, phi, phi, gu)
        A += conv * np.einsum("zq,qk,zqm,zqlm,ca->zkcla", W, phi, uq, G, eye)
    if sigma:
        sym = gu + np.swapaxes(gu, -1, -2)                    # d_m u_c + d_c u_m at [m, c]
        bu -= sigma * (np.einsum("eq,eq,eqkc->ekc", W, pq, G) -
                       mu * np.einsum("eq,eqmc,eqkm->ekc", W, sym, G))
        A += -sigma * mu * (np.einsum("zq,zqkm,zqlm,ca->zkcla", W, G, G, eye) +
                            np.einsum("zq,zqka,zqlc->zkcla", W, G, G))
        Aup += sigma * np.einsum("eq,qj,eqkc->ekcj", W, psi, G)
    if divu:
        div = np.einsum("eqmm->eq", gu)
        bp -= divu * np.einsum("eq,eq,qj->ej", W, div, psi)
        Apu += divu * np.einsum("zq,qj,zqla->zjla", W, psi, G)
    if mass:
        ud = np.einsum("qk,ekn->eqn", phi, np.asarray(udot, np.float64)[adr][:, :d * n2].reshape(-1, n2, d))
        bu -= mass * np.einsum("eq,eqc,qk->ekc", W, ud, phi)
        A += mass * c0 * np.einsum("zq,qk,ql,ca->zkcla", W, phi, phi, eye)
    if source is not None:
        xq = np.einsum("qv,evx->eqx", psi, X)
        f = np.stack(np.broadcast_arrays(*source(*(xq[..., i] for i in range(d)))), -1)
        bu -= np.einsum("eq,eqc,qk->ekc", W, f, phi)
    nu = d * n2
    ae = np.zeros((ne_, nloc, nloc))
    ae[:, :nu, :nu] = A.reshape(ne_, nu, nu)
    ae[:, :nu, nu:] = Aup.reshape(ne_, nu, nv)
    ae[:, nu:, :nu] = Apu.reshape(ne_, nv, nu)
    be = np.concatenate([bu.reshape(ne_, nu), bp], 1)
    mask = np.ones((nloc, nloc), bool)
    mask[nu:, nu:] = False                                    # no pressure-pressure form
    return _scatter(adr, ae, be, n_inc, ia, ja, mask)


def ns_mms_source(x, y):
    """Source of the reference's Navier-Stokes manufactured solution
    u = (x^4 y^4, -4/5 x^3 y^5), p = x^2 y^2 with its sign convention
    (tests/withLinearSolver/navier_stokes.cpp:33-51): f = (u.grad)u + grad p
    - lap u, negated."""
    x, y = np.asarray(x, np.float64), np.asarray(y, np.float64)
    u0, u1 = x ** 4 * y ** 4, -0.8 * x ** 3 * y ** 5
    conv0 = u0 * 4 * x ** 3 * y ** 4 + u1 * 4 * x ** 4 * y ** 3
    conv1 = u0 * (-2.4) * x ** 2 * y ** 5 + u1 * (-4) * x ** 3 * y ** 4
    lap0 = 12 * (x ** 2 * y ** 4 + x ** 4 * y ** 2)
    lap1 = -0.8 * (6 * x * y ** 5 + 20 * x ** 3 * y ** 3)
    return (-(-conv0 - 2 * x * y ** 2 + lap0), -(-conv1 - 2 * x ** 2 * y + lap1))


def l2_error_tet(adr, tet_xyz, u, quad, fct):
    """feNorm L2_ERROR of a scalar P2 field on tetrahedra (src/feNorm.cpp:323-391):
    over the elements in mesh order and the rule's nodes, sum |f - u_h|^2 J w,
    u_h from the element's 10 DOFs (feSpaceTetPn(2) basis), positions from the
    P1 geometry; returns the square root."""
    q = np.asarray(quad, np.float64).reshape(-1, 4)
    X = np.asarray(tet_xyz, np.float64).reshape(-1, 4, 3)
    adr = np.asarray(adr, np.int64).reshape(-1, 10)
    phi, _ = tet_p2_basis(q[:, 0], q[:, 1], q[:, 2])
    psi = np.stack([1 - q[:, 0] - q[:, 1] - q[:, 2], q[:, 0], q[:, 1], q[:, 2]], -1)
    det = np.linalg.det(np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]], -1))
    xq = np.einsum("qv,evx->eqx", psi, X)
    uh = np.asarray(u, np.float64)[adr] @ phi.T
    e2 = (fct(xq[..., 0], xq[..., 1], xq[..., 2]) - uh) ** 2
    return float(np.sqrt(((e2 * q[None, :, 3]).sum(1) * det).sum()))
