"""Oracle set-up: mesh, DOF numbering, element tables, coloring and CSR
pattern of the structured test meshes, restated with numpy.  TEST
INFRASTRUCTURE ONLY: the CPU baseline and the reference arm of bench.py build
their systems with it, so that no part of the product (the CUDA library and
its host set-up) runs on the CPU side; the tests pin every array against the
reference library's own output (tests/golden fixtures).

Restated algorithms:
  * square mesh: n x n cells, each split along the diagonal v00-v11 into
    (v00, v10, v11) and (v00, v11, v01); interior vertices jittered by
    jitter * h * U(-1, 1), two SplitMix64 draws per interior vertex (x then
    y, row-major); boundary lines counter-clockwise from (x0, y0); the
    pressure point is vertex 0.  (The generator of the seeded meshes both
    sides read: the reference has none, its meshes come from files.)
  * edges in order of first appearance over the triangles' local edges
    (k, k+1 mod 3), oriented as first met: the reference reader's edge
    creation order (feMesh2DP1, src/feMeshRead.cpp).
  * numbering feMetaNumber (src/feNumber.cpp:377-427, 677-835): every space
    marks the entities it touches unknown, then every essential space marks
    its entities essential; unknown DOFs first, then essential ones; within
    each, field by field: vertex DOFs in vertex order, then the DOFs of the
    boundary lines (they carry the edge DOFs under them), then edge DOFs in
    edge order.
  * element tables in the layout of feBilinearForm's addressing vectors
    (feSpace::initializeAddressingVector, src/feSpace_2D.cpp): P2 scalar
    [v0 v1 v2 e0 e1 e2]; Taylor-Hood [v0x v0y v1x v1y v2x v2y e0x e0y ...
    e2y p0 p1 p2].
  * coloring feCncGeo::colorElements(1) (src/feCncGeo.cpp:735-790), in C
    (fo_color_elements).
  * CSR pattern feEZCompressedRowStorage (src/feCompressedRowStorage.cpp:15-135):
    the diagonal of every unknown row plus every coupled (row, column) pair of
    the element matrices with both DOFs unknown, sorted and unique per row.
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import sys
from pathlib import Path

import numpy as np


def binding():
    """The oracle's ctypes binding (oracle/oracle.py), loaded from its file:
    with the repository root on sys.path, the name "oracle" can also resolve
    to this directory as a namespace package."""
    mod = sys.modules.get("oracle")
    if mod is not None and hasattr(mod, "load"):
        return mod
    mod = sys.modules.get("fe_oracle_binding")
    if mod is None:
        spec = importlib.util.spec_from_file_location("fe_oracle_binding", Path(__file__).resolve().parent / "oracle.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules["fe_oracle_binding"] = mod
        spec.loader.exec_module(mod)
    return mod


_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64_uniform(seed: int, count: int) -> np.ndarray:
    """The first `count` SplitMix64 outputs of `seed` (Steele, Lea, Flood,
    OOPSLA 2014) mapped to uniform doubles in [-1, 1) with 53 random bits.
    Output k is a function of seed + (k + 1) * gamma alone, so the stream is
    computed as one array."""
    with np.errstate(over="ignore"):
        s = np.uint64(seed) + (np.arange(1, count + 1, dtype=np.uint64) * _GAMMA)
        z = (s ^ (s >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def square_mesh(n: int, x0=0.0, x1=1.0, y0=0.0, y1=1.0, jitter=0.1, seed=1):
    """Vertices (x, y), triangles [nt, 3], boundary lines [nb, 2], pressure point."""
    nv1 = n + 1
    hx, hy = (x1 - x0) / n, (y1 - y0) / n
    i = np.tile(np.arange(nv1), nv1)
    j = np.repeat(np.arange(nv1), nv1)
    x = np.where(i == n, x1, x0 + i.astype(np.float64) * hx)
    y = np.where(j == n, y1, y0 + j.astype(np.float64) * hy)
    interior = (i > 0) & (i < n) & (j > 0) & (j < n)
    if jitter > 0:
        m = int(interior.sum())
        u = splitmix64_uniform(seed, 2 * m)
        x[interior] = x[interior] + (jitter * hx) * u[0::2]
        y[interior] = y[interior] + (jitter * hy) * u[1::2]
    ci, cj = np.meshgrid(np.arange(n), np.arange(n))
    v00 = (cj * nv1 + ci).ravel()
    v10, v01 = v00 + 1, v00 + nv1
    v11 = v01 + 1
    tri = np.stack([v00, v10, v11, v00, v11, v01], 1).reshape(-1, 3).astype(np.int32)
    k = np.arange(n)
    bottom = np.stack([k, k + 1], 1)
    right = np.stack([k * nv1 + n, (k + 1) * nv1 + n], 1)
    top = np.stack([n * nv1 + n - k, n * nv1 + n - k - 1], 1)
    left = np.stack([(n - k) * nv1, (n - k - 1) * nv1], 1)
    bnd = np.concatenate([bottom, right, top, left]).astype(np.int32)
    return x, y, tri, bnd, 0


def edges(tri: np.ndarray, nv: int):
    """tri_edges [nt, 3] (edge k joins local vertices k and k+1) and the edge
    vertices [ne, 2], edges numbered in order of first appearance."""
    a = tri.astype(np.int64)
    b = np.roll(a, -1, axis=1)
    key = (np.minimum(a, b) * nv + np.maximum(a, b)).ravel()
    uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")          # unique keys by first appearance
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    tri_edges = rank[inv].reshape(-1, 3).astype(np.int64)
    ev = np.stack([a.ravel()[first[order]], b.ravel()[first[order]]], 1)
    return tri_edges, ev, (uniq, rank)


def _edge_ids(keys, table):
    uniq, rank = table
    pos = np.searchsorted(uniq, keys)
    if np.any(pos >= len(uniq)) or np.any(uniq[np.minimum(pos, len(uniq) - 1)] != keys):
        raise ValueError("a boundary line is not an edge of the triangulation")
    return rank[pos]


# space: (field, ncomp, degree, support, essential); support "domain" | "boundary" | "point"
def numbering(nv, tri, tri_edges, bnd, bnd_edges, point, spaces):
    """feMetaNumber restated: per field the vertex DOFs vdof[f] [nv, C] and
    edge DOFs edof[f] [ne, C] (-1: none), nInc, nDofs."""
    ne = int(tri_edges.max()) + 1
    nb = len(bnd)
    nf = max(s[0] for s in spaces) + 1
    comp = [0] * nf
    for f, c, _, _, _ in spaces:
        comp[f] = max(comp[f], c)
    NONE, UNK, ESS = 0, 1, 2
    code = [dict(v=np.zeros(nv, np.int8), e=np.zeros(ne, np.int8), l=np.zeros(nb, np.int8)) for _ in range(nf)]

    def mark(s, val):
        f, c, deg, sup, _ = s
        F = code[f]
        if sup == "domain":
            if deg >= 1:
                F["v"][np.unique(tri)] = val
            if deg == 2:
                F["e"][np.unique(tri_edges)] = val
        elif sup == "boundary":
            if deg >= 1:
                F["v"][np.unique(bnd)] = val
            if deg == 2:
                F["l"][:] = val
                F["e"][bnd_edges] = val
        else:
            F["v"][point] = val

    for s in spaces:
        mark(s, UNK)
    for s in spaces:
        if s[4]:
            mark(s, ESS)
    vdof = [np.full((nv, comp[f]), -1, np.int64) for f in range(nf)]
    edof = [np.full((ne, comp[f]), -1, np.int64) for f in range(nf)]
    g = 0
    n_inc = 0
    for want in (UNK, ESS):
        for f in range(nf):
            C_ = comp[f]
            F = code[f]
            vs = np.nonzero(F["v"] == want)[0]
            vdof[f][vs] = g + np.arange(len(vs) * C_).reshape(-1, C_)
            g += len(vs) * C_
            ls = np.nonzero(F["l"] == want)[0]
            es = bnd_edges[ls]
            edof[f][es] = g + np.arange(len(ls) * C_).reshape(-1, C_)
            g += len(ls) * C_
            F["e"][es] = NONE
            eo = np.nonzero(F["e"] == want)[0]
            edof[f][eo] = g + np.arange(len(eo) * C_).reshape(-1, C_)
            g += len(eo) * C_
        if want == UNK:
            n_inc = g
    return vdof, edof, n_inc, g


def element_dofs(tri, tri_edges, vdof, edof, elem_type, fu=0, fp=1):
    if elem_type == 1:
        return np.concatenate([vdof[fu][tri, 0], edof[fu][tri_edges, 0]], 1)
    vu = vdof[fu][tri].reshape(len(tri), 6)
    eu = edof[fu][tri_edges].reshape(len(tri), 6)
    return np.concatenate([vu, eu, vdof[fp][tri, 0]], 1)


def coupling_mask(elem_type):
    if elem_type == 1:
        return np.ones((6, 6), bool)
    i = np.arange(15)
    return (i[:, None] < 12) | (i[None, :] < 12)


def _sorted_unique(a: np.ndarray) -> np.ndarray:
    a = np.sort(a)
    if len(a) == 0:
        return a
    keep = np.empty(len(a), bool)
    keep[0] = True
    np.not_equal(a[1:], a[:-1], out=keep[1:])
    return a[keep]


def csr_pattern(adr: np.ndarray, mask: np.ndarray, n_inc: int):
    """ia [n_inc+1] int64, ja int32: the unknown-row diagonal plus every
    masked coupling of unknown DOFs, sorted and unique per row."""
    ii, jj = np.nonzero(mask)
    chunks = [np.arange(n_inc, dtype=np.int64) * (n_inc + 1)]
    step = max(1, 4_000_000 // max(len(ii), 1))
    for e0 in range(0, len(adr), step):
        a = adr[e0:e0 + step]
        r, c = a[:, ii].ravel(), a[:, jj].ravel()
        keep = (r < n_inc) & (c < n_inc)
        chunks.append(_sorted_unique(r[keep] * n_inc + c[keep]))
    key = _sorted_unique(np.concatenate(chunks))
    rows = key // n_inc
    ja = (key % n_inc).astype(np.int32)
    ia = np.zeros(n_inc + 1, np.int64)
    ia[1:] = np.cumsum(np.bincount(rows, minlength=n_inc))
    return ia, ja


def coloring(tri: np.ndarray, nv: int):
    """Color offsets and elements listed color by color (ascending)."""
    lib = binding().load()
    tri = np.ascontiguousarray(tri, np.int32)
    col = np.empty(len(tri), np.int32)
    nc = lib.fo_color_elements(tri.ctypes.data_as(C.c_void_p), 3, len(tri), nv, col.ctypes.data_as(C.c_void_p))
    if nc < 0:
        raise RuntimeError("coloring failed")
    order = np.argsort(col, kind="stable").astype(np.int32)
    off = np.zeros(nc + 1, np.int64)
    off[1:] = np.cumsum(np.bincount(col, minlength=nc))
    return off, order


class Setup:
    """Everything a CPU solve of one test problem needs."""

    def __init__(self, problem: str, n: int, x0=0.0, x1=1.0, y0=0.0, y1=1.0, jitter=0.1, seed=1):
        x, y, tri, bnd, point = square_mesh(n, x0, x1, y0, y1, jitter, seed)
        nv = len(x)
        tri_edges, ev, table = edges(tri, nv)
        bnd64 = bnd.astype(np.int64)
        bnd_edges = _edge_ids(np.minimum(bnd64[:, 0], bnd64[:, 1]) * nv + np.maximum(bnd64[:, 0], bnd64[:, 1]),
                              table)
        if problem == "diffusion":
            spaces = [(0, 1, 2, "domain", False), (0, 1, 2, "boundary", True)]
            elem_type = 1
        else:
            spaces = [(0, 2, 2, "domain", False), (0, 2, 2, "boundary", True), (1, 1, 1, "domain", False),
                      (1, 1, 1, "point", True)]
            elem_type = 2
        vdof, edof, n_inc, n_dofs = numbering(nv, tri, tri_edges, bnd, bnd_edges, point, spaces)
        self.problem, self.elem_type = problem, elem_type
        self.x, self.y, self.tri, self.bnd, self.point = x, y, tri, bnd, point
        self.tri_edges, self.edge_v = tri_edges, ev
        self.vdof, self.edof = vdof, edof
        self.n_inc, self.n_dofs = n_inc, n_dofs
        self.adr = np.ascontiguousarray(element_dofs(tri, tri_edges, vdof, edof, elem_type), np.int64)
        self.ia, self.ja = csr_pattern(self.adr, coupling_mask(elem_type), n_inc)
        self.color_offsets, self.color_elements = coloring(tri, nv)
        self.elem_xy = np.stack([x[tri[:, 0]], y[tri[:, 0]], x[tri[:, 1]], y[tri[:, 1]], x[tri[:, 2]],
                                 y[tri[:, 2]]], 1)

    def dof_positions(self):
        """(x, y, field, component) of every DOF; edge DOFs at the midpoint."""
        xs = np.zeros(self.n_dofs)
        ys = np.zeros(self.n_dofs)
        fld = np.zeros(self.n_dofs, np.int32)
        cmp_ = np.zeros(self.n_dofs, np.int32)
        mx = 0.5 * (self.x[self.edge_v[:, 0]] + self.x[self.edge_v[:, 1]])
        my = 0.5 * (self.y[self.edge_v[:, 0]] + self.y[self.edge_v[:, 1]])
        for f, (vd, ed) in enumerate(zip(self.vdof, self.edof)):
            for c in range(vd.shape[1]):
                for d, px, py in ((vd[:, c], self.x, self.y), (ed[:, c], mx, my)):
                    ok = d >= 0
                    xs[d[ok]] = px[ok]
                    ys[d[ok]] = py[ok]
                    fld[d[ok]] = f
                    cmp_[d[ok]] = c
        return xs, ys, fld, cmp_
