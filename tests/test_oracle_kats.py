"""Pins the CPU oracle against the reference's own known-answer tests and checks
the committed golden fixtures reproduce (CPU only)."""
from pathlib import Path

import numpy as np
import pytest

import gridap_oracle as go
from helpers import make_problem

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_local_range_matches_divrem_rule():
    # PArraysExtras.jl:72-84: last `rem` parts get one more cell; ghost layer clamped
    assert [go.local_range(p, 3, 10) for p in (1, 2, 3)] == [(0, 3), (3, 6), (6, 10)]
    assert go.local_range(2, 3, 10, ghost=True) == (2, 7)
    assert go.local_range(1, 1, 5, ghost=True) == (0, 5)


def test_ghost_maps_and_perm():
    P = go.make_partition((2, 2), (4, 4))
    g2g, g2o, perm = P.ghost_maps(0)
    # part 0 owns cells [0,2)x[0,2) and sees a 1-cell halo: 9 local cells, 5 ghosts
    assert len(perm) == 9 and sorted(perm.tolist()) == list(range(9))
    assert len(g2g) == 5 and set(g2o.tolist()) == {1, 2, 3}


@pytest.mark.parametrize("parts", [(1, 1), (1, 2), (2, 1), (2, 2)])
def test_dof_count_4x4_q1(parts):
    # test/sequential/PeriodicBCsTests.jl:7-20, non-periodic case: 25 free DOFs
    pb = go.Problem(np=parts, n=(4, 4), domain=(0, 1, 0, 1), order=1, dirichlet_sides=(0, 0, 0, 0))
    fe = go.build_fespace(pb)
    assert fe.dofs[0].ngdofs == 25


@pytest.mark.parametrize("strategy", ["sub", "full"])
@pytest.mark.parametrize("parts", [(2, 2), (1, 1), (2, 1), (1, 2)])
def test_fespaces_q1_solution_kat(parts, strategy):
    # test/FESpacesTests.jl:10-59: Q1, u=x+y, error < 1e-9
    pb = make_problem(2, (4, 4), parts, 1, f=0.0, u=lambda x, y: x + y, domain=(0, 4, 0, 4))
    pb.degree = 3
    fe = go.build_fespace(pb)
    mats = go.assemble(pb, fe, strategy)
    for M in mats:   # FESpacesTests.jl:29-31 local matrix size == local index sets
        assert (M.nrows, M.ncols) == (len(M.row_own_gids) + len(M.row_ghost_gids),
                                      len(M.col_own_gids) + len(M.col_ghost_gids))
    x = go.solve_lu(mats, fe.dofs[0].ngdofs)
    e = go.l2_error(pb, go.nodal_solution(pb, fe, x), lambda x, y: x + y)
    assert e < 1e-9


@pytest.mark.parametrize("strategy", ["sub", "full"])
def test_vector_kat_sum_b(strategy):
    # test/FESpacesTests.jl:61-70: ∫(1*v) on (0,4)^2 4x4 Q1 -> sum(b) == length(b)
    pb = go.Problem(np=(2, 2), n=(4, 4), domain=(0, 4, 0, 4), order=1, degree=3, f_const=1.0)
    fe = go.build_fespace(pb)
    A, b = go.gather_global(go.assemble(pb, fe, strategy), fe.dofs[0].ngdofs)
    assert abs(b.sum() - len(b)) < 1e-12


@pytest.mark.parametrize("strategy", ["sub", "full"])
def test_poisson_q2_kat(strategy):
    # test/PoissonTests.jl:14-45 (Dirichlet on the whole boundary): Q2 reproduces (x+y)^2
    pb = make_problem(2, (4, 4), (2, 2), 2, f=-4.0, u=lambda x, y: (x + y) ** 2, domain=(0, 4, 0, 4))
    fe = go.build_fespace(pb)
    x = go.solve_lu(go.assemble(pb, fe, strategy), fe.dofs[0].ngdofs)
    assert go.l2_error(pb, go.nodal_solution(pb, fe, x), lambda x, y: (x + y) ** 2) < 1e-9


def test_measure_kat():
    # test/CellDataTests.jl:48: ∫(1)dΩ ≈ 16 on (0,4)^2
    pb = go.Problem(np=(2, 2), n=(4, 4), domain=(0, 4, 0, 4), order=1, degree=2)
    _, _, F = go.reference_matrices(2, 1, pb.h, 2)
    assert abs(F.sum() * 16 - 16.0) < 1e-12


def test_strategies_agree_on_global_system():
    pb = make_problem(3, (5, 4, 3), (2, 2, 1), 1, seed=3)
    fe = go.build_fespace(pb)
    A, b = go.gather_global(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    Af, bf = go.gather_global(go.assemble(pb, fe, "full"), fe.dofs[0].ngdofs)
    assert abs(A - Af).max() < 1e-14 and np.abs(b - bf).max() < 1e-14


def test_pcg_matches_lu():
    pb = make_problem(3, (6, 6, 6), (2, 2, 2), 1, seed=0)
    fe = go.build_fespace(pb)
    mats = go.assemble(pb, fe, "sub")
    A, b = go.gather_global(mats, fe.dofs[0].ngdofs)
    x1 = go.solve_lu(mats, fe.dofs[0].ngdofs)
    x2, _ = go.pcg_jacobi(A, b, 1e-13)
    assert np.abs(x1 - x2).max() / np.abs(x1).max() < 1e-8


@pytest.mark.parametrize("fixture", sorted(GOLDEN.glob("*.npz")), ids=lambda p: p.stem)
def test_golden_fixture_reproduces(fixture):
    import make_golden as mg
    name, strategy = fixture.stem.rsplit("_", 1)
    pb = make_problem(**mg.CASES[name])
    fe = go.build_fespace(pb)
    mats = go.assemble(pb, fe, strategy)
    g = np.load(fixture)
    for p, (d, M) in enumerate(zip(fe.dofs, mats)):
        assert np.array_equal(g[f"p{p}_gid"], d.ldof_to_gdof)
        assert np.array_equal(g[f"p{p}_owner"], d.ldof_to_owner)
        assert np.array_equal(g[f"p{p}_rowptr"], M.rowptr)
        assert np.array_equal(g[f"p{p}_colidx"], M.colidx)
        assert np.array_equal(g[f"p{p}_gcol_gid"], M.col_ghost_gids)
        assert np.allclose(g[f"p{p}_vals"], M.vals, rtol=0, atol=1e-13)
        assert np.allclose(g[f"p{p}_b"], M.b, rtol=0, atol=1e-13)


def test_c1_q2_128_solution_kat():
    """The C1 configuration at full size (2D Q2, 128^2 cells, parts (2,2), degree 4,
    u = (x+y)^2 on the boundary, f = -4): the known answer of test/PoissonTests.jl:14-45
    holds for the oracle's assembly and gathered LU at the size the GPU parity test uses
    (L2 error < 1e-9; the discretisation reproduces (x+y)^2 exactly)."""
    u = lambda x, y: (x + y) ** 2
    pb = make_problem(2, (128, 128), (2, 2), 2, f=-4.0, u=u)
    fe = go.build_fespace(pb)
    assert fe.dofs[0].ngdofs == 255 * 255
    x = go.solve_lu(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    assert go.l2_error(pb, go.nodal_solution(pb, fe, x), u) < 1e-9
