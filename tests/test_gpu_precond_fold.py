"""The folded saddle-point preconditioner against the unfolded one.

The steady two-component preconditioner applies the pressure block and the
velocity right-hand side without a separate pressure pass: with
z_p = sc r_p + c u (c the pressure sum) the velocity V-cycle input is
b0 - c G u, and the V-cycle is linear, so the result is V(b0) - c V(G u) with
V(G u) formed once per Jacobian.  FENG_PFOLD=0 keeps the unfolded
sequence (pressure sum, pressure block, velocity right-hand side, V-cycle).
Both must give the same Newton solution on the 64 x 64 Kovasznay mesh (its
finest multigrid level is large enough for the sliced-ELL kernels that
carry the fold), FP64 and mixed, with FGMRES iteration counts within a few
percent of each other."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SNIPPET = r"""
import json, sys
import numpy as np
from feng_gb300 import api as fe, kovasznay
_, num, forms = kovasznay.build(64)
sys_, sol = kovasznay.make_system(num, forms, sys.argv[1])
st = fe.solveNewtonRaphson(sys_, sol, kovasznay.newton_options(sys.argv[1]))
np.save(sys.argv[2], sys_.getSolution())
print(json.dumps({"return": st["return"], "krylov": st.get("krylov_iterations", -1)}))
"""


def _run(precision, fold, out):
    env = dict(os.environ)
    env["FENG_PFOLD"] = "1" if fold else "0"
    r = subprocess.run([sys.executable, "-c", SNIPPET, precision, str(out)], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_folded_preconditioner_matches_unfolded(precision, tmp_path):
    a = _run(precision, True, tmp_path / "fold.npy")
    b = _run(precision, False, tmp_path / "plain.npy")
    assert a["return"] == 0 and b["return"] == 0, (a, b)
    ua, ub = np.load(tmp_path / "fold.npy"), np.load(tmp_path / "plain.npy")
    assert np.max(np.abs(ua - ub)) <= 1e-7 * np.max(np.abs(ub))
    if a["krylov"] >= 0 and b["krylov"] >= 0:
        assert abs(a["krylov"] - b["krylov"]) <= max(3, 0.05 * b["krylov"]), (a, b)

