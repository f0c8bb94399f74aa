"""Essential-component constraints and periodicity: the oracle's
restatement of feLinearSystemMklPardiso::constrainEssentialComponents /
applyPeriodicity (src/feLinearSystemMklPardiso.cpp:994-1149) against an
independent numpy statement of the same rules, on the reference's CSR
pattern (golden fixture).  The MKL backend itself cannot be built here (no
MKL), so this row is pinned by restatement only."""
import numpy as np

from conftest import load_golden
from oracle import oracle as orc


def _numpy_rules(ia, ja, values, rhs, rows, master, slave):
    v, r = values.copy(), rhs.copy()
    n = len(ia) - 1
    rows = [x for x in rows if 0 <= x < n]
    for row in rows:                      # columns first
        v[ja == row] = 0.0
    for row in rows:                      # then the rows, 1 on the diagonal
        seg = slice(ia[row], ia[row + 1])
        v[seg] = np.where(ja[seg] == row, 1.0, 0.0)
        r[row] = 0.0
    for m, s in zip(master, slave):
        if not (0 <= m < n and 0 <= s < n):
            continue
        seg = slice(ia[s], ia[s + 1])
        v[seg] = np.where(ja[seg] == s, 1.0, np.where(ja[seg] == m, -1.0, 0.0))
        r[s] = 0.0
    return v, r


def test_oracle_matches_numpy_statement():
    g = load_golden("kovasznay_th_8")
    ia, ja = g["ia"], g["ja"]
    n = len(ia) - 1
    rng = np.random.default_rng(4)
    values = rng.normal(size=len(ja))
    rhs = rng.normal(size=n)
    rows = rng.choice(n, 25, replace=False).tolist() + [n + 5, -1]   # out-of-range entries ignored
    master = rng.choice(n, 6, replace=False)
    slave = (master + 7) % n
    v1, r1 = orc.constrain(ia, ja, values, rhs, rows, master, slave)
    v2, r2 = _numpy_rules(ia, ja.astype(np.int64), values, rhs, rows, master, slave)
    np.testing.assert_array_equal(v1, v2)
    np.testing.assert_array_equal(r1, r2)
