"""The drop-in feLinearSystemCUDA (feng_gb300/adapter) compiles against the
reference's own headers and links with the reference library and the CUDA
backend (where the reference checkout and its library build are present)."""
import os
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT, reference_root

REF = reference_root() or Path("/nonexistent")
LIBREF = ROOT / "oracle" / "_ref" / "libfeNG.a"


@pytest.mark.skipif(not (REF / "src" / "feLinearSystem.h").exists() or not LIBREF.exists(),
                    reason="reference checkout or its library build not present")
def test_dropin_adapter_builds_against_reference(tmp_path, built_library):
    exe = tmp_path / "kovasznay_dropin"
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-DHAVE_OMP", "-DHAVE_EIGEN", "-w",
           f"-I{REF / 'src'}", "-isystem", str(REF / "contrib" / "eigen"), "-isystem", str(REF / "contrib" / "gmsh"),
           f"-I{ROOT / 'include'}", f"-I{ROOT / 'feng_gb300' / 'adapter'}",
           str(ROOT / "tests" / "adapter" / "kovasznay_dropin.cpp"), str(LIBREF), str(built_library),
           f"-Wl,-rpath,{built_library.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert exe.exists()
