"""Python mirror of feNG's operator API for the hot path.

Names, argument order and meaning follow the reference so that a driver
reads like feNG's own tests (tests/withLinearSolver/*.cpp):

    mesh = Mesh2DP1.generate_square(64, jitter=0.1, seed=1)
    u  = createFiniteElementSpace(mesh, LAGRANGE, 2, "U", "Domaine", 4, zero)
    uB = createFiniteElementSpace(mesh, LAGRANGE, 2, "U", "Bord", 4, exact)
    numbering = feMetaNumber(mesh, [uB, u], [uB])
    diff = createBilinearForm([u], feSysElm_Diffusion(1.0))
    src  = createBilinearForm([u], feSysElm_Source(SRC_SIN_SIN, [-2 pi^2]))
    system = createLinearSystem(CUDA, [diff, src], numbering, options)
    sol = feSolution(system)
    sol.initializeEssentialBC()
    stats = solveNewtonRaphson(system, sol, feNLSolverOptions(...))

Every compute call goes through the C ABI of include/feng_cuda.h into the
CUDA backend; nothing here computes element matrices or solves.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import check, ptr

LAGRANGE = "LAGRANGE"
VECTOR_LAGRANGE = "VECTOR_LAGRANGE"
CUDA = "CUDA"

CNC = {"Domaine": 0, "Bord": 1, "PointPression": 2}

# Form kinds (FE_FORM_* in include/feng_cuda.h)
SOURCE, DIFFUSION, VECTOR_SOURCE, TRANSIENT_VECTOR_MASS = 1, 2, 3, 4
MIXED_DIVERGENCE, VECTOR_CONVECTIVE_ACCELERATION, DIV_NEWTONIAN_STRESS = 5, 6, 7
# Device source registry (FE_SRC_*)
SRC_NONE, SRC_SIN_SIN, SRC_NS_MMS_POLY, SRC_CONST_VEC, SRC_SIN_BODY = 0, 1, 2, 3, 4
SRC_SIN3, SRC_SIN3_BODY = 5, 6   # tetrahedra
ELEM_P2, ELEM_TAYLOR_HOOD, ELEM_TET_P2, ELEM_TET_TAYLOR_HOOD = 1, 2, 3, 4


class Mesh2DP1:
    """Triangle mesh with physical groups "Domaine", "Bord", "PointPression"."""

    def __init__(self, handle):
        self._h = handle
        self._lib = _lib.load()

    @classmethod
    def generate_square(cls, n: int, x0=0.0, x1=1.0, y0=0.0, y1=1.0, jitter=0.1, seed=1):
        lib = _lib.load()
        h = C.c_void_p()
        check(lib.fe_mesh_generate_square(n, x0, x1, y0, y1, jitter, seed, C.byref(h)))
        return cls(h)

    @classmethod
    def from_msh(cls, path: str, domain: str = "Domaine", boundary: Sequence[str] = ("Bord",),
                 point: str | None = "PointPression"):
        """Reads an ASCII msh 4.1 file.  `domain`, `boundary` and `point` name
        the file's physical groups taken as "Domaine" (triangles), "Bord"
        (the lines of all listed groups) and "PointPression" (None: none)."""
        lib = _lib.load()
        h = C.c_void_p()
        if domain == "Domaine" and tuple(boundary) == ("Bord",) and point == "PointPression":
            check(lib.fe_mesh_read_msh(str(path).encode(), C.byref(h)))
        else:
            names = (C.c_char_p * max(len(boundary), 1))(*[b.encode() for b in boundary])
            check(lib.fe_mesh_read_msh_groups(str(path).encode(), domain.encode(), names, len(boundary),
                                              None if point is None else point.encode(), C.byref(h)))
        return cls(h)

    @classmethod
    def from_arrays(cls, x, y, tri, bnd, point=-1):
        """Mesh from vertex coordinates, counter-clockwise triangles ("Domaine"),
        boundary lines ("Bord") and the "PointPression" vertex (-1: none)."""
        lib = _lib.load()
        x = np.ascontiguousarray(x, np.float64); y = np.ascontiguousarray(y, np.float64)
        tri = np.ascontiguousarray(tri, np.int32).reshape(-1); bnd = np.ascontiguousarray(bnd, np.int32).reshape(-1)
        h = C.c_void_p()
        check(lib.fe_mesh_from_arrays(len(x), ptr(x), ptr(y), len(tri) // 3, ptr(tri), len(bnd) // 2, ptr(bnd),
                                      int(point), C.byref(h)))
        return cls(h)

    def write_msh(self, path: str):
        check(self._lib.fe_mesh_write_msh(self._h, str(path).encode()))

    def sizes(self):
        nv, nt, ne, nb = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(self._lib.fe_mesh_sizes(self._h, C.byref(nv), C.byref(nt), C.byref(ne), C.byref(nb)))
        return nv.value, nt.value, ne.value, nb.value

    def arrays(self):
        nv, nt, ne, nb = self.sizes()
        x = np.empty(nv); y = np.empty(nv)
        tri = np.empty(3 * nt, np.int32); te = np.empty(3 * nt, np.int32)
        bnd = np.empty(2 * nb, np.int32); pt = np.empty(1, np.int32)
        check(self._lib.fe_mesh_arrays(self._h, ptr(x), ptr(y), ptr(tri), ptr(te), ptr(bnd), ptr(pt)))
        return dict(x=x, y=y, tri=tri.reshape(-1, 3), tri_edges=te.reshape(-1, 3),
                    bnd=bnd.reshape(-1, 2), point=int(pt[0]), n_edges=ne)

    def getNumElements(self):
        return self.sizes()[1]

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            self._lib.fe_mesh_destroy(h)


class Mesh3DP1:
    """Tetrahedral mesh with physical groups "Domaine" (tetrahedra) and
    "Bord" (boundary triangles), read by the reference as feMesh2DP1."""

    def __init__(self, handle):
        self._h = handle
        self._lib = _lib.load()

    @classmethod
    def generate_cube(cls, n: int, x0=0.0, x1=1.0, y0=0.0, y1=1.0, z0=0.0, z1=1.0, jitter=0.05, seed=1):
        """n^3 cells, 6 Kuhn tetrahedra each, interior vertices jittered by
        U(-jitter h, jitter h) per axis (SplitMix64 seeded with `seed`)."""
        lib = _lib.load()
        box = np.array([x0, x1, y0, y1, z0, z1], np.float64)
        h = C.c_void_p()
        check(lib.fe_mesh3d_generate_cube(n, ptr(box), jitter, seed, C.byref(h)))
        return cls(h)

    @classmethod
    def from_msh(cls, path: str):
        """Reads the "Domaine" tetrahedra and "Bord" triangles of a msh 4.1 file."""
        lib = _lib.load()
        h = C.c_void_p()
        check(lib.fe_mesh3d_read_msh(str(path).encode(), C.byref(h)))
        return cls(h)

    @classmethod
    def from_arrays(cls, x, y, z, tet, bnd):
        lib = _lib.load()
        x, y, z = (np.ascontiguousarray(v, np.float64) for v in (x, y, z))
        tet = np.ascontiguousarray(tet, np.int32).reshape(-1)
        bnd = np.ascontiguousarray(bnd, np.int32).reshape(-1)
        h = C.c_void_p()
        check(lib.fe_mesh3d_from_arrays(len(x), ptr(x), ptr(y), ptr(z), len(tet) // 4, ptr(tet), len(bnd) // 3,
                                        ptr(bnd), C.byref(h)))
        return cls(h)

    def write_msh(self, path: str):
        check(self._lib.fe_mesh3d_write_msh(self._h, str(path).encode()))

    def sizes(self):
        nv, nt, nb = C.c_int64(), C.c_int64(), C.c_int64()
        check(self._lib.fe_mesh3d_sizes(self._h, C.byref(nv), C.byref(nt), C.byref(nb)))
        return nv.value, nt.value, nb.value

    def arrays(self):
        nv, nt, nb = self.sizes()
        x, y, z = np.empty(nv), np.empty(nv), np.empty(nv)
        tet, bnd = np.empty(4 * nt, np.int32), np.empty(3 * nb, np.int32)
        check(self._lib.fe_mesh3d_arrays(self._h, ptr(x), ptr(y), ptr(z), ptr(tet), ptr(bnd)))
        return dict(x=x, y=y, z=z, tet=tet.reshape(-1, 4), bnd=bnd.reshape(-1, 3))

    def getNumElements(self):
        return self.sizes()[1]

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            self._lib.fe_mesh3d_destroy(h)


@dataclass
class feSpace:
    mesh: Mesh2DP1
    element: str
    degree: int
    fieldID: str
    cncGeoID: str
    degreeQuadrature: int
    fct: Optional[Callable] = None

    @property
    def ncomp(self):
        if self.element != VECTOR_LAGRANGE:
            return 1
        return 3 if isinstance(self.mesh, Mesh3DP1) else 2


def createFiniteElementSpace(mesh, element, degree, fieldID, cncGeoID, degreeQuadrature, fct=None):
    """createFiniteElementSpace (src/feSpace.cpp:11-420) for the spaces the
    backend supports: Lagrange P1/P2 (scalar or 2-vector) on "Domaine" and
    "Bord", P0 on "PointPression"."""
    if cncGeoID not in CNC:
        raise ValueError(f"unknown connectivity {cncGeoID!r}")
    if element not in (LAGRANGE, VECTOR_LAGRANGE):
        raise ValueError(f"unsupported element {element!r}")
    deg = 0 if cncGeoID == "PointPression" else degree
    return feSpace(mesh, element, deg, fieldID, cncGeoID, degreeQuadrature, fct)


class feMetaNumber:
    """DOF numbering of feMetaNumber (src/feNumber.cpp:677-835)."""

    def __init__(self, mesh, spaces: Sequence[feSpace], essentialSpaces: Sequence[feSpace]):
        self.mesh = mesh
        self.spaces = list(spaces)
        self.essentialSpaces = list(essentialSpaces)
        self.fieldIDs = []
        for s in self.spaces:
            if s.fieldID not in self.fieldIDs:
                self.fieldIDs.append(s.fieldID)
        for e in self.essentialSpaces:
            if not any(e is s for s in self.spaces):
                raise ValueError("every essential space must be listed among the spaces")
        arr = (_lib.SpaceDesc * len(self.spaces))()
        for i, s in enumerate(self.spaces):
            arr[i] = _lib.SpaceDesc(self.fieldIDs.index(s.fieldID), s.degree, s.ncomp, CNC[s.cncGeoID],
                                    int(any(s is e for e in self.essentialSpaces)))
        self._desc = arr
        dom = [s for s in self.spaces if s.cncGeoID == "Domaine"]
        vector = any(s.element == VECTOR_LAGRANGE and s.degree == 2 for s in dom)
        if isinstance(mesh, Mesh3DP1):
            self.elem_type = ELEM_TET_TAYLOR_HOOD if vector else ELEM_TET_P2
        else:
            self.elem_type = ELEM_TAYLOR_HOOD if vector else ELEM_P2
        qdeg = {s.degreeQuadrature for s in dom}
        if len(qdeg) != 1:
            raise ValueError("the domain spaces must share one quadrature degree")
        self.quad_degree = qdeg.pop()
        self._setups = {}
        st = self.setup()
        self.nInc, self.nDofs = st.nInc, st.nDofs

    def setup(self, pc_block_rows: int = 256) -> "feSetup":
        """Host tables (numbering, element DOFs, coloring, pattern) for the backend."""
        if pc_block_rows not in self._setups:
            self._setups[pc_block_rows] = feSetup(self, pc_block_rows)
        return self._setups[pc_block_rows]

    def getNbUnknowns(self):
        return self.nInc

    def getNbDOFs(self):
        return self.nDofs


def setPatternMode(mode: int):
    """Where set-ups build the CSR pattern: -1 the CUDA device when one is
    present (default), 0 the host threads, 1 the device."""
    check(_lib.load().fe_setup_set_pattern_mode(int(mode)))


class feSetup:
    """Set-up of the standalone route (fe_setup_* in include/feng_cuda.h):
    host threads, the CSR pattern on the device when one is present; needs
    no GPU."""

    def __init__(self, numbering: feMetaNumber, pc_block_rows: int = 256):
        self.lib = _lib.load()
        self.numbering = numbering
        h = C.c_void_p()
        if isinstance(numbering.mesh, Mesh3DP1):
            check(self.lib.fe_setup3d_create(numbering.mesh._h, C.cast(numbering._desc, C.c_void_p),
                                             len(numbering.spaces), numbering.elem_type, pc_block_rows,
                                             C.byref(h)))
        else:
            check(self.lib.fe_setup_create(numbering.mesh._h, C.cast(numbering._desc, C.c_void_p),
                                           len(numbering.spaces), numbering.elem_type,
                                           numbering.quad_degree, pc_block_rows, C.byref(h)))
        self._h = h
        n = [C.c_int64() for _ in range(4)]
        nc, nl = C.c_int(), C.c_int()
        check(self.lib.fe_setup_sizes(h, *[C.byref(v) for v in n], C.byref(nc), C.byref(nl)))
        self.nInc, self.nDofs, self.nnz, self.nElm = (v.value for v in n)
        self.nColors, self.nloc = nc.value, nl.value

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            self.lib.fe_setup_destroy(h)

    def pattern(self):
        ia = np.empty(self.nInc + 1, np.int64)
        ja = np.empty(self.nnz, np.int32)
        check(self.lib.fe_setup_get_pattern(self._h, ptr(ia), ptr(ja)))
        return ia, ja

    @property
    def patternOnDevice(self) -> bool:
        v = C.c_int()
        check(self.lib.fe_setup_pattern_on_device(self._h, C.byref(v)))
        return bool(v.value)

    def coloring(self):
        off = np.empty(self.nColors + 1, np.int64)
        el = np.empty(self.nElm, np.int32)
        check(self.lib.fe_setup_get_coloring(self._h, ptr(off), ptr(el)))
        return off, el

    def elementDofs(self):
        adr = np.empty(self.nElm * self.nloc, np.int64)
        check(self.lib.fe_setup_get_element_dofs(self._h, ptr(adr)))
        return adr.reshape(self.nElm, self.nloc)

    def dofInfo(self):
        x = np.empty(self.nDofs); y = np.empty(self.nDofs)
        f = np.empty(self.nDofs, np.int32); c = np.empty(self.nDofs, np.int32)
        v = np.empty(self.nDofs, np.int32)
        check(self.lib.fe_setup_get_dof_info(self._h, ptr(x), ptr(y), ptr(f), ptr(c), ptr(v)))
        return x, y, f, c, v

    def dofZ(self):
        """z coordinate of every DOF (tetrahedral meshes)."""
        z = np.empty(self.nDofs)
        check(self.lib.fe_setup_get_dof_z(self._h, ptr(z)))
        return z

    def blocks(self):
        b = np.empty(self.nInc, np.int32)
        check(self.lib.fe_setup_get_blocks(self._h, ptr(b)))
        return b


def quadrature_rule(degree: int):
    """(r, s, w) of the triangle rule of the given degree."""
    lib = _lib.load()
    n = C.c_int()
    r, s, w = np.empty(16), np.empty(16), np.empty(16)
    check(lib.fe_quadrature_rule(degree, C.byref(n), ptr(r), ptr(s), ptr(w)))
    k = n.value
    return r[:k].copy(), s[:k].copy(), w[:k].copy()


def tet_quadrature_rule(degree: int):
    """Symmetric tetrahedral rule of the given degree (1..8): r, s, t, w."""
    lib = _lib.load()
    n = C.c_int()
    check(lib.fe_tet_quadrature_rule(degree, C.byref(n), None, None, None, None))
    r, s, t, w = (np.empty(n.value) for _ in range(4))
    check(lib.fe_tet_quadrature_rule(degree, C.byref(n), ptr(r), ptr(s), ptr(t), ptr(w)))
    return r, s, t, w


@dataclass
class feSysElm:
    kind: int
    coeff: float = 1.0
    coeff2: float = 0.0
    source: int = SRC_NONE
    params: tuple = (0.0, 0.0, 0.0, 0.0)


def feSysElm_Diffusion(coeff=1.0):
    return feSysElm(DIFFUSION, coeff)


def feSysElm_Source(source=SRC_SIN_SIN, params=(1.0,), coeff=1.0):
    return feSysElm(SOURCE, coeff, 0.0, source, tuple(params) + (0.0,) * (4 - len(params)))


def feSysElm_VectorSource(source=SRC_NS_MMS_POLY, params=(), coeff=1.0):
    return feSysElm(VECTOR_SOURCE, coeff, 0.0, source, tuple(params) + (0.0,) * (4 - len(params)))


def feSysElm_VectorConvectiveAcceleration(coeff=1.0):
    return feSysElm(VECTOR_CONVECTIVE_ACCELERATION, coeff)


def feSysElm_MixedDivergence(coeff=1.0):
    return feSysElm(MIXED_DIVERGENCE, coeff)


def feSysElm_DivergenceNewtonianStress(coeff=1.0, viscosity=1.0):
    return feSysElm(DIV_NEWTONIAN_STRESS, coeff, viscosity)


def feSysElm_TransientVectorMass(coeff=1.0):
    return feSysElm(TRANSIENT_VECTOR_MASS, coeff)


@dataclass
class feBilinearForm:
    spaces: list
    sysElm: feSysElm


def createBilinearForm(spaces, sysElm):
    return feBilinearForm(list(spaces), sysElm)


@dataclass
class LinearSolverOptions:
    krylov: str = "fgmres"        # "cg" | "fgmres"
    restart: int = 50
    max_iter: int = 10000
    rel_tol: float = 1e-8         # feLinearSystem::_rel_tol (src/feLinearSystem.h:66)
    abs_tol: float = 1e-14
    div_tol: float = 1e6
    precond: str = "amg"           # "none" | "bjacobi-ilu0" | "ilu0" | "jacobi" | "amg"
    pc_block_rows: int = 256
    precision: str = "fp64"       # "fp64" | "mixed"
    mg_inner: int = 0             # multigrid: inner AMG-CG steps per velocity component
    mg_smooth: int = 1            # multigrid: Chebyshev smoother degree
    gs_passes: int = 1            # mixed FGMRES Gram-Schmidt: 1 adaptive (second pass when needed), 2 always twice,
                                  # 3 adaptive with the norm of the update by Pythagoras

    def to_c(self, quad_degree: int) -> _lib.Options:
        pc = {"none": 0, "bjacobi-ilu0": 1, "ilu0": 1, "jacobi": 2, "amg": 3}[self.precond]
        rows = 0 if self.precond == "ilu0" else self.pc_block_rows
        return _lib.Options(0 if self.krylov == "cg" else 1, self.restart, self.max_iter, self.rel_tol,
                            self.abs_tol, self.div_tol, pc, rows,
                            1 if self.precision == "mixed" else 0, quad_degree, self.mg_inner,
                            self.mg_smooth, self.gs_passes)


class feLinearSystemCUDA:
    """The CUDA backend behind the feLinearSystem interface
    (src/feLinearSystem.h:43-169)."""

    def __init__(self, forms: Sequence[feBilinearForm], numbering: feMetaNumber,
                 options: LinearSolverOptions | None = None, rule=None):
        """rule: optional quadrature rule rows (r, s, [t,] w) replacing the one
        of the spaces' degree (e.g. the reference's tabulated values); it is
        kept by the numbering's set-up for later systems too."""
        self.lib = _lib.load()
        self.forms = list(forms)
        self.numbering = numbering
        self.options = options or LinearSolverOptions()
        self.elem_type = numbering.elem_type
        qdeg = {s.degreeQuadrature for f in self.forms for s in f.spaces}
        if qdeg != {numbering.quad_degree}:
            raise ValueError("all forms must use the quadrature rule of the domain spaces")
        self.quad_degree = numbering.quad_degree
        rows = 0 if self.options.precond == "ilu0" else self.options.pc_block_rows
        self.setup = numbering.setup(rows)
        if rule is not None:
            r = np.ascontiguousarray(rule, np.float64)
            check(self.lib.fe_setup_set_quadrature(self.setup._h, len(r), ptr(r)))
        fa = (_lib.FormDesc * len(self.forms))()
        for i, f in enumerate(self.forms):
            se = f.sysElm
            fa[i] = _lib.FormDesc(se.kind, se.coeff, se.coeff2, se.source, (C.c_double * 4)(*se.params))
        opts = self.options.to_c(self.quad_degree)
        h = C.c_void_p()
        check(self.lib.fe_cuda_system_create(self.setup._h, C.cast(fa, C.c_void_p), len(self.forms),
                                             C.byref(opts), C.byref(h)))
        self._h = h
        n = [C.c_int64() for _ in range(4)]
        nc = C.c_int()
        check(self.lib.fe_cuda_system_sizes(h, *[C.byref(v) for v in n], C.byref(nc)))
        self.nInc, self.nDofs, self.nnz, self.nElm = (v.value for v in n)
        self.nColors = nc.value

    # feLinearSystem::constrainEssentialComponents / applyPeriodicity
    # (src/feLinearSystemMklPardiso.cpp:994-1149)
    def setConstrainedRows(self, rows):
        rows = np.ascontiguousarray(rows, np.int64)
        check(self.lib.fe_cuda_set_constrained_rows(self._h, ptr(rows), len(rows)))

    def constrainEssentialComponents(self):
        check(self.lib.fe_cuda_constrain_essential_components(self._h))

    def setPeriodicPairs(self, master, slave):
        master = np.ascontiguousarray(master, np.int64)
        slave = np.ascontiguousarray(slave, np.int64)
        if master.shape != slave.shape:
            raise ValueError("master and slave lists differ in length")
        check(self.lib.fe_cuda_set_periodic_pairs(self._h, ptr(master), ptr(slave), len(master)))

    def applyPeriodicity(self):
        check(self.lib.fe_cuda_apply_periodicity(self._h))

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            self.lib.fe_cuda_system_destroy(h)

    # -- feLinearSystem operations
    def getSystemSize(self):
        return self.nInc

    def setToZero(self):
        check(self.lib.fe_cuda_set_to_zero(self._h))

    def setMatrixToZero(self):
        check(self.lib.fe_cuda_set_matrix_to_zero(self._h))

    def setResidualToZero(self):
        check(self.lib.fe_cuda_set_residual_to_zero(self._h))

    def assembleResiduals(self):
        check(self.lib.fe_cuda_assemble_residuals(self._h))

    def assembleMatrices(self):
        check(self.lib.fe_cuda_assemble_matrices(self._h))

    def assemble(self):
        self.assembleMatrices()
        self.assembleResiduals()

    def getRHSMaxNorm(self):
        v = C.c_double()
        check(self.lib.fe_cuda_get_rhs_max_norm(self._h, C.byref(v)))
        return v.value

    def setTolerances(self, rel_tol=None, abs_tol=None, max_iter=None):
        """setRelativeTol / setAbsoluteTol / setMaxIter (src/feLinearSystem.h:86-89)."""
        o = self.options
        o.rel_tol = o.rel_tol if rel_tol is None else rel_tol
        o.abs_tol = o.abs_tol if abs_tol is None else abs_tol
        o.max_iter = o.max_iter if max_iter is None else max_iter
        check(self.lib.fe_cuda_set_tolerances(self._h, o.rel_tol, o.abs_tol, o.max_iter))

    def solve(self, raise_on_failure=True):
        dx, rhs, axb, it = C.c_double(), C.c_double(), C.c_double(), C.c_int()
        s = self.lib.fe_cuda_solve(self._h, C.byref(dx), C.byref(rhs), C.byref(axb), C.byref(it))
        if raise_on_failure:
            check(s)
        return dict(status=s, normDx=dx.value, normRHS=rhs.value, normAxb=axb.value,
                    nIter=it.value)

    def applyPreconditioner(self, r):
        """z = M^-1 r with the current preconditioner (PETSc's PCApply)."""
        r = np.ascontiguousarray(r, np.float64)
        z = np.empty(self.nInc)
        check(self.lib.fe_cuda_apply_preconditioner(self._h, ptr(r), ptr(z)))
        return z

    def correctSolution(self):
        check(self.lib.fe_cuda_correct_solution(self._h))

    # -- state
    def setSolution(self, u, udot=None):
        u = np.ascontiguousarray(u, np.float64)
        ud = None if udot is None else np.ascontiguousarray(udot, np.float64)
        check(self.lib.fe_cuda_set_solution(self._h, ptr(u), ptr(ud)))

    def getSolution(self):
        u = np.empty(self.nDofs)
        check(self.lib.fe_cuda_get_solution(self._h, ptr(u)))
        return u

    def setTime(self, t, c0=0.0):
        check(self.lib.fe_cuda_set_time(self._h, t, c0))

    def setBDF(self, order, cn, hist1=None, hist2=None):
        cn = np.ascontiguousarray(np.resize(np.asarray(cn, np.float64), 3))
        h1 = None if hist1 is None else np.ascontiguousarray(hist1, np.float64)
        h2 = None if hist2 is None else np.ascontiguousarray(hist2, np.float64)
        check(self.lib.fe_cuda_set_bdf(self._h, order, ptr(cn), ptr(h1), ptr(h2)))

    # -- views for checks
    def getMatrix(self):
        v = np.empty(self.nnz)
        check(self.lib.fe_cuda_get_matrix(self._h, ptr(v)))
        return v

    def getRHS(self):
        v = np.empty(self.nInc)
        check(self.lib.fe_cuda_get_rhs(self._h, ptr(v)))
        return v

    def getDu(self):
        v = np.empty(self.nInc)
        check(self.lib.fe_cuda_get_du(self._h, ptr(v)))
        return v

    @property
    def jacobianRoute(self):
        """1: row-owned Jacobian assembly, 0: colored scatter."""
        r = C.c_int()
        check(self.lib.fe_cuda_jacobian_route(self._h, C.byref(r)))
        return r.value

    def getResidualMaxNorm(self):
        """max |du| of the last correction, reduced on the device
        (feLinearSystem::getResidualMaxNorm)."""
        n = C.c_double()
        check(self.lib.fe_cuda_get_du_max_norm(self._h, C.byref(n)))
        return n.value

    def pattern(self):
        ia = np.empty(self.nInc + 1, np.int64)
        ja = np.empty(self.nnz, np.int32)
        check(self.lib.fe_cuda_get_pattern(self._h, ptr(ia), ptr(ja)))
        return ia, ja

    def coloring(self):
        off = np.empty(self.nColors + 1, np.int64)
        el = np.empty(self.nElm, np.int32)
        check(self.lib.fe_cuda_get_coloring(self._h, ptr(off), ptr(el)))
        return off, el

    def elementDofs(self):
        return self.setup.elementDofs()

    def dofInfo(self):
        return self.setup.dofInfo()[:4]

    def times(self):
        v = [C.c_double() for _ in range(4)]
        check(self.lib.fe_cuda_get_times(self._h, *[C.byref(t) for t in v]))
        return dict(zip(("residual_ms", "matrix_ms", "factor_ms", "solve_ms"), (t.value for t in v)))

    def resetTimes(self):
        check(self.lib.fe_cuda_reset_times(self._h))

    def synchronize(self):
        check(self.lib.fe_cuda_synchronize(self._h))


def createLinearSystem(kind, forms, numbering, options: LinearSolverOptions | None = None, rule=None):
    if kind != CUDA:
        raise ValueError("only the CUDA backend is provided")
    return feLinearSystemCUDA(forms, numbering, options, rule)


class feSolution:
    """Host view of the solution vector; the authoritative copy lives on the device."""

    def __init__(self, system: feLinearSystemCUDA):
        self.system = system
        self.u = np.zeros(system.nDofs)
        self.udot = np.zeros(system.nDofs)
        self.t = 0.0
        self.c0 = 0.0
        self.dof_x, self.dof_y, self.dof_field, self.dof_comp = system.dofInfo()
        self.dof_z = system.setup.dofZ() if isinstance(system.numbering.mesh, Mesh3DP1) else None

    def initializeEssentialBC(self, t: float = 0.0):
        """Nodewise essential values (feSolution::initializeEssentialBC,
        src/feSolution.cpp:246-...): the function of each field's essential
        space evaluated at the DOF locations (vertices, edge midpoints)."""
        num = self.system.numbering
        ess = np.arange(self.system.nInc, self.system.nDofs)
        for fi, fid in enumerate(num.fieldIDs):
            spaces = [s for s in num.essentialSpaces if s.fieldID == fid and s.fct is not None]
            if not spaces:
                continue
            sel = ess[self.dof_field[ess] == fi]
            for s in spaces:
                xyz = (self.dof_x[sel], self.dof_y[sel]) + (() if self.dof_z is None else (self.dof_z[sel],))
                vals = s.fct(*xyz)
                comp = self.dof_comp[sel]
                out = np.empty(len(sel))
                for c in range(len(vals)):
                    m = comp == c
                    out[m] = np.broadcast_to(vals[c], sel.shape)[m]
                self.u[sel] = out
                break
        self.push()

    def push(self):
        self.system.setSolution(self.u, self.udot)

    def pull(self):
        self.u = self.system.getSolution()
        return self.u


# ---- visualisation export (src/feExporter.h, src/feExporter.cpp) -----------------

VTK = "VTK"


class feExporterVTK:
    """feExporterVTK (src/feExporter.h:68-98): writes the solution as the
    reference's legacy ASCII VTK file (fe_export_vtk), on the host.  `sol` is
    a feSolution (its device copy is read) or an array of every DOF."""

    def __init__(self, numbering: feMetaNumber, sol, mesh: Mesh2DP1, spaces: Sequence[feSpace]):
        self.numbering, self.sol, self.mesh = numbering, sol, mesh
        self.spaces = list(spaces)

    def writeStep(self, fileName, requiredFields: Sequence[str] = (), precision: int = 6):
        """writeStep (src/feExporter.cpp:854-990): the fields of the domain
        spaces (those named in requiredFields, if any); `precision`
        significant digits (the reference writes 6)."""
        num = self.numbering
        u = self.sol.pull() if isinstance(self.sol, feSolution) else self.sol
        u = np.ascontiguousarray(u, np.float64)
        if u.shape != (num.nDofs,):
            raise ValueError(f"the solution must hold {num.nDofs} DOFs")
        wanted = [s.fieldID for s in self.spaces if s.cncGeoID == "Domaine"]
        if requiredFields:
            wanted = [f for f in wanted if f in requiredFields]
        if not wanted:
            raise ValueError("no field of a domain space to export")
        names = (C.c_char_p * len(num.fieldIDs))(*[f.encode() for f in num.fieldIDs])
        req = (C.c_char_p * len(wanted))(*[f.encode() for f in wanted])
        st = num.setup()
        lib = _lib.load()
        fn = lib.fe_export_vtk3d if isinstance(self.mesh, Mesh3DP1) else lib.fe_export_vtk
        check(fn(self.mesh._h, st._h, ptr(u), names, len(num.fieldIDs), req, len(wanted), int(precision),
                 str(fileName).encode()))


def createVisualizationExporter(fmt, numbering, solution, mesh, spaces):
    """createVisualizationExporter (src/feExporter.cpp:65-77) for VTK."""
    if fmt != VTK:
        raise ValueError(f"unsupported visualization format {fmt!r}")
    return feExporterVTK(numbering, solution, mesh, spaces)


# ---- error norms (src/feNorm.h, src/feNorm.cpp) ---------------------------------

L2_ERROR, VECTOR_L2_ERROR = "L2_ERROR", "VECTOR_L2_ERROR"


class feNorm:
    """L2_ERROR / VECTOR_L2_ERROR of feNorm (src/feNorm.cpp:152-163, 323-391,
    1399-1443): the exact solution is evaluated on the host at the nodes of
    the system's quadrature rule on every element (once per compute, as the
    reference's feFunction calls), the error integral runs on the device from
    the device solution."""

    def __init__(self, normType, spaces, sol: feSolution, scalarSolution=None, vectorSolution=None):
        if normType not in (L2_ERROR, VECTOR_L2_ERROR):
            raise ValueError(f"unsupported norm {normType!r}")
        space = spaces[0]
        vector = space.element == VECTOR_LAGRANGE
        if (normType == VECTOR_L2_ERROR) != vector:
            raise ValueError("VECTOR_L2_ERROR needs a vector space, L2_ERROR a scalar one")
        fct = vectorSolution if vector else scalarSolution
        if fct is None:
            raise ValueError("the error norm needs the exact solution")
        self.system = sol.system
        taylor_hood = self.system.elem_type == ELEM_TAYLOR_HOOD
        if taylor_hood:
            if vector and space.degree == 2:
                self.field = 0
            elif not vector and space.degree == 1:
                self.field = 1
            else:
                raise ValueError("Taylor-Hood systems hold a P2 vector field and a P1 scalar field")
        elif not vector and space.degree == 2:
            self.field = 0
        else:
            raise ValueError("scalar P2 systems hold one P2 scalar field")
        self.ncomp = 2 if vector else 1
        self.fct = fct
        self.sol = sol

    def points(self):
        """Quadrature nodes (x, y) of every element, shape (nElm, nq)."""
        lib, h = self.system.lib, self.system._h
        nq = C.c_int()
        check(lib.fe_cuda_norm_points(h, C.byref(nq), None, None))
        x = np.empty(self.system.nElm * nq.value)
        y = np.empty_like(x)
        check(lib.fe_cuda_norm_points(h, C.byref(nq), ptr(x), ptr(y)))
        return x.reshape(-1, nq.value), y.reshape(-1, nq.value)

    def compute(self) -> float:
        x, y = self.points()
        vals = self.fct(x.ravel(), y.ravel())
        ex = np.empty((x.size, self.ncomp))
        for c in range(self.ncomp):
            ex[:, c] = np.broadcast_to(vals[c], x.size)
        ex = np.ascontiguousarray(ex)
        err = C.c_double()
        check(self.system.lib.fe_cuda_l2_error(self.system._h, self.field, ptr(ex), C.byref(err)))
        return err.value


def createNorm(normType, spaces, sol, scalarSolution=None, vectorSolution=None):
    """createNorm (src/feNorm.cpp:7-...) for the L2 error norms."""
    return feNorm(normType, spaces, sol, scalarSolution, vectorSolution)


@dataclass
class feNLSolverOptions:
    tolResidual: float = 1e-10
    tolCorrection: float = 1e-10
    tolDivergence: float = 1e4
    maxIter: int = 20
    recomputeJacobianEveryNsteps: int = 3
    residualDecrease: float = 1e-1
    relResidual: float = 0.0
    linearRtolMin: float = 0.0
    residualScale: float = 0.0


def solveNewtonRaphson(system: feLinearSystemCUDA, sol: feSolution | None,
                       tol: feNLSolverOptions, stationary: bool = True):
    """solveNewtonRaphson (src/feNonLinearSolver.cpp:38-181) on device data."""
    if sol is not None:
        sol.push()
    o = _lib.NewtonOptions(tol.tolResidual, tol.tolCorrection, tol.tolDivergence, int(tol.maxIter),
                           tol.recomputeJacobianEveryNsteps, tol.residualDecrease, int(stationary),
                           tol.relResidual, tol.linearRtolMin, tol.residualScale)
    st = _lib.NewtonStats()
    s = system.lib.fe_cuda_newton(system._h, C.byref(o), C.byref(st))
    out = {k: getattr(st, k) for k, _ in _lib.NewtonStats._fields_}
    out["return"] = s
    if sol is not None:
        sol.pull()
    if s not in (0, -5):
        check(s)
    return out


# ---- time integration (src/feTimeIntegration.h) --------------------------------

BDF2 = "BDF2"
GUESS = {"previous": 0, "extrapolate": 1, "learned": 2}


class BDF2Integrator:
    """BDF2Integrator (src/feTimeIntegration.cpp:449-547) on device-resident
    history: the first step starts with a BDF1 substep of 0.1 dt
    (startWithBDF1, :383-435), then variable-step BDF2.  ``guess`` picks the
    Newton initial guess of each step: "previous" (the reference's),
    "extrapolate" (linear in time) or "learned" (extrapolation plus an online
    trained per-node MLP correction, used only where its FP64 residual is
    smaller).  Each Newton solve stops at ||R||inf <= relResidual * ||R(u^n)||inf
    (plus the absolute tests of ``nlOptions``)."""

    def __init__(self, system: feLinearSystemCUDA, sol: feSolution | None, nlOptions: feNLSolverOptions,
                 t0: float, t1: float, nTimeSteps: int, guess: str = "extrapolate", trainFrom: int = 20,
                 useFrom: int = 25, trainIters: int = 8, batch: int = 16384, lr: float = 1e-3, seed: int = 1):
        self.system, self.sol = system, sol
        self.dt = (t1 - t0) / nTimeSteps
        if sol is not None:
            sol.push()
        o = _lib.TransientOptions(self.dt, t0, GUESS[guess], trainFrom, useFrom, trainIters, batch, lr, seed)
        n = _lib.NewtonOptions(nlOptions.tolResidual, nlOptions.tolCorrection, nlOptions.tolDivergence,
                               int(nlOptions.maxIter), nlOptions.recomputeJacobianEveryNsteps,
                               nlOptions.residualDecrease, 0, nlOptions.relResidual, nlOptions.linearRtolMin, 0.0)
        h = C.c_void_p()
        check(system.lib.fe_cuda_transient_create(system._h, C.byref(o), C.byref(n), C.byref(h)))
        self._h = h

    def makeSteps(self, nSteps: int, raise_on_failure: bool = True):
        """Advances nSteps steps; returns one statistics dict per step.  A step
        whose Newton solve fails stops the run: FeError is raised, or with
        raise_on_failure=False the steps done so far are returned, the last
        one carrying the failure in "status"."""
        st = (_lib.StepStats * max(nSteps, 1))()
        s = self.system.lib.fe_cuda_transient_steps(self._h, nSteps, C.cast(st, C.c_void_p))
        if raise_on_failure:
            check(s)
        if self.sol is not None:
            self.sol.pull()
        return [{k: getattr(x, k) for k, _ in _lib.StepStats._fields_} for x in st[:nSteps] if x.step > 0]

    def getNetwork(self) -> np.ndarray:
        """The learned guess's network parameters (float32, fe_mlp packing)."""
        n = C.c_int64()
        d = [C.c_int() for _ in range(4)]
        check(self.system.lib.fe_mlp_sizes(*[C.byref(v) for v in d], C.byref(n)))
        out = np.empty(n.value, np.float32)
        check(self.system.lib.fe_cuda_transient_get_network(self._h, ptr(out)))
        return out

    def setNetwork(self, params):
        """Warm-starts the learned guess from saved parameters."""
        p = np.ascontiguousarray(params, np.float32)
        check(self.system.lib.fe_cuda_transient_set_network(self._h, ptr(p)))

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            self.system.lib.fe_cuda_transient_destroy(h)


def createTimeIntegrator(scheme: str, nlOptions: feNLSolverOptions, system: feLinearSystemCUDA,
                         sol: feSolution | None, t0: float, t1: float, nTimeSteps: int, **kw):
    """createTimeIntegrator (src/feTimeIntegration.cpp) for the BDF2 scheme."""
    if scheme != BDF2:
        raise ValueError("only the BDF2 scheme runs on the device")
    return BDF2Integrator(system, sol, nlOptions, t0, t1, nTimeSteps, **kw)


class MLP:
    """The learned-guess network alone (device kernels, host buffers)."""

    def __init__(self, seed: int = 1, max_batch: int = 4096):
        self.lib = _lib.load()
        d = [C.c_int() for _ in range(4)]
        npar = C.c_int64()
        check(self.lib.fe_mlp_sizes(*[C.byref(v) for v in d], C.byref(npar)))
        self.dims = tuple(v.value for v in d)
        self.nparams = npar.value
        h = C.c_void_p()
        check(self.lib.fe_mlp_create(seed, max_batch, C.byref(h)))
        self._h = h

    def params(self) -> np.ndarray:
        p = np.empty(self.nparams, np.float32)
        check(self.lib.fe_mlp_get_params(self._h, ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(self.lib.fe_mlp_set_params(self._h, ptr(p)))

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty((x.shape[0], self.dims[3]), np.float32)
        check(self.lib.fe_mlp_forward(self._h, ptr(x), x.shape[0], ptr(y)))
        return y

    def train_step(self, x, t, mask, lr):
        """Gradient and loss of the batch, then one Adam step; returns (loss, grad)."""
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        mask = np.ascontiguousarray(mask, np.float32)
        g = np.empty(self.nparams, np.float32)
        loss = C.c_double()
        check(self.lib.fe_mlp_train_step(self._h, ptr(x), ptr(t), ptr(mask), x.shape[0], lr, ptr(g),
                                         C.byref(loss)))
        return loss.value, g

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            self.lib.fe_mlp_destroy(h)
