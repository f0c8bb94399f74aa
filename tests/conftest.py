import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session", autouse=True)
def built_library():
    """Builds the in-tree CUDA library once (nvcc cross-compiles without a GPU)."""
    from feng_gb300 import build
    build.build()
    return build.LIB


def reference_root():
    """The reference checkout (CPU tests that read it skip without it):
    FENG_REFERENCE, else the location the build recorded when it compiled
    the reference library into oracle/_ref; None when neither exists."""
    import os
    env = os.environ.get("FENG_REFERENCE")
    if env:
        return Path(env) if Path(env).exists() else None
    rec = ROOT / "oracle" / "_ref" / "REFERENCE"
    if rec.exists():
        p = Path(rec.read_text().strip())
        return p if p.exists() else None
    return None


def load_golden(name):
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def golden_names(transient=False):
    """Fixture names of the triangle cases: the steady cases (assembly state
    + Newton solution), or the BDF2 runs with transient=True.  Tetrahedral
    fixtures (key "tet") and the probes of large cases (key "sha_ia") have
    their own tests."""
    out = []
    for p in sorted(GOLDEN.glob("*.npz")):
        with np.load(p) as z:
            if "tet" in z.files or "sha_ia" in z.files:   # tetrahedra / probes of large cases
                continue
            if ("steps" in z.files) == transient:
                out.append(p.stem)
    return out
