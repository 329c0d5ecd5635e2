"""Failure detection without a GPU fault: the grid-barrier waits of the persistent kernels
are bounded.  A probe launches blocks that wait for one arrival more than there are
blocks (a flag that nothing sets): every wait runs out after the given limit, the kernel
returns, the host reads GD_ERR_TIMEOUT, and the context stays usable -- the barrier with
all arrivals passes, and a mixed-precision solve (the persistent kernel) afterwards
matches the oracle."""
import time

import ctypes as C
import numpy as np
import pytest

import gridap_oracle as go
from helpers import make_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    import gridap_gb300 as G
    be = G.GB300Backend(0)
    yield be
    be.close()


def probe(backend, blocks, expected, timeout_s):
    from gridap_gb300 import _lib as L
    return L.load().gd_debug_barrier_probe(backend.handle, blocks, expected, C.c_double(timeout_s))


def test_barrier_wait_runs_out_and_context_survives(backend):
    import gridap_gb300 as G
    from gridap_gb300 import _lib as L
    assert probe(backend, 4, 4, 0.5) == 0                       # every arrival comes: passes
    for blocks in (1, 3):
        t0 = time.perf_counter()
        st = probe(backend, blocks, blocks + 1, 0.25)           # one arrival never comes
        dt = time.perf_counter() - t0
        assert st == 4, L.load().gd_last_error()                # GD_ERR_TIMEOUT
        assert 0.2 < dt < 2.0
    assert probe(backend, 8, 8, 0.5) == 0                       # the context is still usable
    # and the persistent solver still runs and is correct
    case = dict(dim=3, n=(9, 8, 7), parts=(2, 2, 1), order=1, seed=44, domain=(0, 1.125, 0, 1.0, 0, 0.875))
    pb = make_problem(**case)
    fe = go.build_fespace(pb)
    x_ref = go.solve_lu(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    ranks = backend.distribute(range(int(np.prod(pb.np))))
    model = G.CartesianDiscreteModel(ranks, pb.np, pb.domain, pb.n)
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, 1), dirichlet_tags="boundary")
    U = G.TrialFESpace(0.0, V)
    dO = G.Measure(G.Triangulation(model), pb.degree)
    op = G.AffineFEOperator(G.integral_grad_grad(pb.kappa, dO), G.integral_source(pb.f_const, dO), U, V)
    x = op.matrix.solve(rtol=1e-12, method="mixed_ir")
    assert op.matrix.last_stats.converged
    assert np.abs(x - x_ref).max() / np.abs(x_ref).max() <= 1e-8


def test_probe_rejects_bad_arguments(backend):
    assert probe(backend, 0, 1, 0.1) == 1                       # GD_ERR_ARG
    assert probe(backend, 2, 2, 10.0) == 1                      # limit above 5 s
