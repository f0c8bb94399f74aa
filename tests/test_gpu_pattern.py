"""CSR pattern built on the device (fe_pattern.cu) against the host builder
(build_csr_pattern, the reference's feEZCompressedRowStorage rule): the same
row pointers and column indices, bit for bit, on triangles and tetrahedra,
scalar P2 and Taylor-Hood, with and without essential DOFs."""
import numpy as np
import pytest

import feng_gb300 as fe
from feng_gb300 import cube, kovasznay

pytestmark = pytest.mark.gpu


def _numberings():
    out = []
    _, num, _ = kovasznay.build(24, 40.0)
    out.append(("kovasznay_24", num))
    _, num3, _ = cube.build(5, 100.0)
    out.append(("cube_th_5", num3))
    m3 = fe.Mesh3DP1.generate_cube(6, jitter=0.05, seed=2)
    u = fe.createFiniteElementSpace(m3, fe.LAGRANGE, 2, "U", "Domaine", 4)
    uB = fe.createFiniteElementSpace(m3, fe.LAGRANGE, 2, "U", "Bord", 4)
    out.append(("cube_p2_6", fe.feMetaNumber(m3, [uB, u], [uB])))
    return out


@pytest.mark.parametrize("case", range(3))
def test_device_pattern_equals_host(case):
    name, num = _numberings()[case]
    try:
        fe.setPatternMode(0)
        host = fe.feSetup(num)
        assert not host.patternOnDevice
        fe.setPatternMode(1)
        dev = fe.feSetup(num)
        assert dev.patternOnDevice
    finally:
        fe.setPatternMode(-1)
    ia_h, ja_h = host.pattern()
    ia_d, ja_d = dev.pattern()
    np.testing.assert_array_equal(ia_d, ia_h, err_msg=name)
    np.testing.assert_array_equal(ja_d, ja_h, err_msg=name)
    # the default (automatic) mode takes the device here
    assert fe.feSetup(num).patternOnDevice
