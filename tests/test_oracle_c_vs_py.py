"""The oracle's C restatement (oracle/oracle_core.c) against its Python restatement.

oracle_core.c is the timed CPU baseline of bench.py (the reference arm and the
cpu_baseline leg), so it must assemble what the Python oracle assembles: per part the
local CSR pattern (rowptr, colidx), the ghost rows and ghost columns (gids, in the
reference's order) bit-exact, values within 1e-12 x max|row| and the right-hand side
within 1e-12 x max|b| (the two sum the same COO triplets; only the quadrature's
rounding may differ).  Cases: the Q1 golden problems, both strategies, 2D and 3D, with a
random cell-wise kappa, partial Dirichlet sides, and a 3D Q1 case with (2,2,2) parts
like the bench workload.  CPU only.
"""
import numpy as np
import pytest

import gridap_oracle as go
import oracle_c
from helpers import make_problem, row_scaled_error

CASES = [
    # dim, cells, parts, sides (None = whole boundary), seed
    (2, (4, 4), (2, 2), None, 1),
    (2, (7, 5), (3, 2), None, 2),
    (2, (6, 6), (2, 1), (1, 0, 0, 1), 3),
    (3, (6, 5, 4), (2, 2, 2), None, 4),
    (3, (9, 8, 7), (2, 2, 2), None, 5),
    (3, (5, 6, 7), (3, 1, 2), (1, 0, 1, 0, 0, 1), 6),
]


def _compare(pb, strategy):
    fe = go.build_fespace(pb)
    ref = go.assemble(pb, fe, strategy)
    sides = pb.dirichlet_sides if pb.dirichlet_sides is not None else (1,) * (2 * pb.dim)
    got, _, _ = oracle_c.assemble(pb.dim, pb.n, pb.np, pb.domain, sides, pb.kappa, pb.f_const, pb.degree,
                                  strategy, threads=1, keep=True)
    assert len(got) == len(ref)
    for p, (M, C) in enumerate(zip(ref, got)):
        assert np.array_equal(C["rowptr"], M.rowptr), f"part {p}: rowptr"
        assert np.array_equal(C["colidx"], M.colidx), f"part {p}: colidx"
        assert np.array_equal(C["row_ghost_gids"], M.row_ghost_gids), f"part {p}: ghost rows"
        assert np.array_equal(C["col_ghost_gids"], M.col_ghost_gids), f"part {p}: ghost columns"
        assert row_scaled_error(C["vals"], M.vals, M.rowptr) <= 1e-12, f"part {p}: values"
        bscale = max(np.abs(M.b).max(), 1e-300) if len(M.b) else 1.0
        assert np.abs(C["b"] - M.b).max(initial=0.0) <= 1e-12 * bscale, f"part {p}: rhs"


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}d-{'x'.join(map(str, c[1]))}-p{'x'.join(map(str, c[2]))}"
                                             for c in CASES])
@pytest.mark.parametrize("strategy", ["sub", "full"])
def test_oracle_c_matches_python_oracle(case, strategy):
    dim, n, parts, sides, seed = case
    pb = make_problem(dim, n, parts, 1, sides=sides, seed=seed)
    _compare(pb, strategy)


def test_oracle_c_matches_python_oracle_without_kappa():
    pb = make_problem(3, (4, 4, 4), (2, 2, 1), 1, seed=None)
    _compare(pb, "sub")
