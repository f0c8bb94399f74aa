"""Builders of device systems used by the GPU tests."""
import ctypes as C

import numpy as np

import feng_gb300 as fe
from feng_gb300 import _lib
from feng_gb300._lib import check, ptr


class TablesSystem(fe.api.feLinearSystemCUDA):
    """A system created through the drop-in route (fe_cuda_system_create_from_tables)
    from the reference's own tables: element DOFs, CSR pattern, coloring."""

    def __init__(self, g, forms, options):  # noqa: D401 - no super().__init__
        """g: the tables (fixture keys); on tetrahedra "tet" and "xyz" (the
        four vertices' x y z per element), and optionally "quad_rule" (rows
        r, s, [t,] w) to use instead of the rule of the options' degree."""
        self.lib = _lib.load()
        self.options = options
        if "tet" in g:
            tri = g["tet"]
            nloc = g["adr"].size // len(tri)
            elem_type = fe.api.ELEM_TET_P2 if nloc == 10 else fe.api.ELEM_TET_TAYLOR_HOOD
            xy = np.ascontiguousarray(g["xyz"], np.float64).reshape(len(tri), 12)
        else:
            tri = g["tri"]
            elem_type = 1 if g["adr"].size // len(tri) == 6 else 2
            xy = np.empty((len(tri), 6))
            for k in range(3):
                xy[:, 2 * k] = g["x"][tri[:, k]]
                xy[:, 2 * k + 1] = g["y"][tri[:, k]]
        self.elem_type = elem_type
        self._keep = [np.ascontiguousarray(a) for a in
                      (g["adr"].astype(np.int64), xy, g["color_offsets"].astype(np.int64),
                       g["color_elements"].astype(np.int32), g["ia"].astype(np.int64),
                       g["ja"].astype(np.int32))]
        adr, xy, off, el, ia, ja = self._keep
        fa = (_lib.FormDesc * len(forms))()
        for i, f in enumerate(forms):
            se = f.sysElm
            fa[i] = _lib.FormDesc(se.kind, se.coeff, se.coeff2, se.source, (C.c_double * 4)(*se.params))
        opts = options.to_c(int(g["quad_degree"]))
        h = C.c_void_p()
        rule = None if g.get("quad_rule") is None else np.ascontiguousarray(g["quad_rule"], np.float64)
        check(self.lib.fe_cuda_system_create_from_tables_rule(
            elem_type, len(tri), ptr(adr), ptr(xy), int(g["nInc"]), int(g["nDofs"]), len(off) - 1,
            ptr(off), ptr(el), ptr(ia), ptr(ja), None, C.cast(fa, C.c_void_p), len(forms),
            C.byref(opts), 0 if rule is None else len(rule), ptr(rule), C.byref(h)))
        self._h = h
        n = [C.c_int64() for _ in range(4)]
        nc = C.c_int()
        check(self.lib.fe_cuda_system_sizes(h, *[C.byref(v) for v in n], C.byref(nc)))
        self.nInc, self.nDofs, self.nnz, self.nElm = (v.value for v in n)
        self.nColors = nc.value
