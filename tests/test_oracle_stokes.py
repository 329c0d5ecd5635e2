"""The oracle's restatement of the multi-field test with fields on different spaces
(test/MultiFieldTests.jl:14-57: vector Q2 velocity, discontinuous P1 pressure with the
zero-mean constraint, a Stokes form), checked on the CPU against that test's known
answers: the L2 errors of the solved velocity and pressure below 1e-9.  Also: the
corrected pressure has zero mean, and the result does not depend on which pressure DOF
the zero-mean space fixes (the mean correction removes the constant)."""
import numpy as np
import pytest

import stokes_oracle as so


def _case(domain):
    x0, x1, y0, y1 = domain
    mean = 0.5 * (x0 + x1) + 0.5 * (y0 + y1)   # mean of x + y over the rectangle
    u = lambda x, y: ((x + y) ** 2, (x - y) ** 2)
    p = lambda x, y: x + y - mean
    f = lambda x, y: (-4.0 + 1.0, -4.0 + 1.0)   # -lap u + grad p
    g = lambda x, y: 4.0 * y                     # div u
    return u, p, f, g


@pytest.mark.parametrize("n,domain", [((4, 4), (0.0, 4.0, 0.0, 4.0)),        # the reference test's mesh
                                      ((6, 5), (0.0, 1.5, -1.0, 0.25))],
                         ids=["reference_4x4", "rect_6x5"])
def test_stokes_known_answer(n, domain):
    u, p, f, g = _case(domain)
    S = so.stokes_system(n, domain, 2, u, p, f, g)
    uv, pv = so.stokes_solve(S)
    eu, ep = so.stokes_l2_errors(S, uv, pv, u, p)
    assert eu < 1e-9 and ep < 1e-9
    assert abs(float(pv @ S.dvol)) <= 1e-12 * S.vol   # zero mean after the correction


def test_stokes_mean_correction_is_independent_of_the_fixed_dof():
    """Fixing another pressure DOF (the first, or one in the middle) gives the same velocity
    and, after the mean correction, the same pressure."""
    domain = (0.0, 4.0, 0.0, 4.0)
    u, p, f, g = _case(domain)
    S = so.stokes_system((4, 4), domain, 2, u, p, f, g)
    uv, pv = so.stokes_solve(S)
    for other in (0, 23):
        T = so.stokes_system((4, 4), domain, 2, u, p, f, g, p_fixed=other)
        uv2, pv2 = so.stokes_solve(T)
        assert np.abs(uv2 - uv).max() <= 1e-11 * np.abs(uv).max()
        assert np.abs(pv2 - pv).max() <= 1e-11 * np.abs(pv).max()
