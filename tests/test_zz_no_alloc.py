"""The allocation-free max-norm entry point (fe_cuda_max_norm_noalloc) gives
the same value as the regular fe_cuda_get_rhs_max_norm on the same residual,
on two calls in a row, through the C ABI.

It exists for callers that may not allocate device memory (a framework that
owns every device byte through its own pool, or a loop that cannot afford
cudaMalloc's implicit synchronization); its scratch is a static device array
of the library.  This file is collected last so that a failure here does not
hide the other tests; it also passes when run alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

import feng_gb300 as fe
from conftest import load_golden
from feng_gb300 import _lib
from helpers import golden_mesh, problem_spaces

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the tolerance of the FP64 parity tests (a max-norm is exact in practice)


def test_noalloc_max_norm_matches_regular_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    lib = _lib.load()
    g = load_golden("kovasznay_th_8")
    num, forms = problem_spaces("ns_kovasznay", golden_mesh(g), 40.0)
    sys = fe.createLinearSystem(fe.CUDA, forms, num, fe.LinearSolverOptions(precond="ilu0"))
    sys.setSolution(g["u0"])
    sys.setToZero()
    sys.assembleResiduals()
    sys.synchronize()
    expected = sys.getRHSMaxNorm()           # regular entry point (allocated scratch)
    rhs = sys.getRHS()
    assert expected > 0 and np.isclose(expected, np.max(np.abs(rhs)), rtol=0, atol=0)

    # The caller owns the input: a device copy of the residual made by torch.
    x = torch.from_numpy(rhs).to("cuda:0")
    torch.cuda.synchronize()
    # A first call loads the kernel's module (and with it the static scratch)
    # if nothing had; after it, the device's free memory must not move.
    out = C.c_double(-1.0)
    assert lib.fe_cuda_max_norm_noalloc(C.c_void_p(x.data_ptr()), x.numel(), None, C.byref(out)) == 0
    free_before = torch.cuda.mem_get_info(0)[0]
    for _ in range(2):                        # two calls in a row share the static scratch
        out = C.c_double(-1.0)
        s = lib.fe_cuda_max_norm_noalloc(C.c_void_p(x.data_ptr()), x.numel(), None, C.byref(out))
        assert s == 0, lib.fe_cuda_last_error()
        assert abs(out.value - expected) <= TOL * expected
    assert torch.cuda.mem_get_info(0)[0] == free_before, "the entry point allocated device memory"

    # Sizes beyond the static scratch are rejected before any work.
    out = C.c_double(-1.0)
    s = lib.fe_cuda_max_norm_noalloc(C.c_void_p(x.data_ptr()), 4194304 + 1, None, C.byref(out))
    assert s == -3 and b"exceed the maximum" in lib.fe_cuda_last_error()
