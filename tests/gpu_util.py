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
        self.lib = _lib.load()
        self.options = options
        elem_type = 1 if g["adr"].size // len(g["tri"]) == 6 else 2
        self.elem_type = elem_type
        nloc = 6 if elem_type == 1 else 15
        tri = g["tri"]
        xy = np.empty((len(tri), 6))
        for k in range(3):
            xy[:, 2 * k] = g["x"][tri[:, k]]
            xy[:, 2 * k + 1] = g["y"][tri[:, k]]
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
        check(self.lib.fe_cuda_system_create_from_tables(
            elem_type, len(tri), ptr(adr), ptr(xy), int(g["nInc"]), int(g["nDofs"]), len(off) - 1,
            ptr(off), ptr(el), ptr(ia), ptr(ja), None, C.cast(fa, C.c_void_p), len(forms),
            C.byref(opts), C.byref(h)))
        self._h = h
        n = [C.c_int64() for _ in range(4)]
        nc = C.c_int()
        check(self.lib.fe_cuda_system_sizes(h, *[C.byref(v) for v in n], C.byref(nc)))
        self.nInc, self.nDofs, self.nnz, self.nElm = (v.value for v in n)
        self.nColors = nc.value
