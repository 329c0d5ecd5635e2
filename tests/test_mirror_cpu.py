"""Host-side checks of the Python mirror that need no GPU: the reference-API calls whose
options the device does not implement are refused with NotImplementedError (there is no
CPU fallback), before any device work."""
import pytest


def test_reference_fe_p_space_is_refused():
    import gridap_gb300 as G
    assert G.ReferenceFE(G.lagrangian, float, 2) == ("lagrangian", float, 2)
    assert G.ReferenceFE(G.lagrangian, float, 1, space=":Q") == ("lagrangian", float, 1)
    with pytest.raises(NotImplementedError):
        G.ReferenceFE(G.lagrangian, float, 1, space=":P")


def test_zero_mean_constraint_is_refused():
    import gridap_gb300 as G
    reffe = G.ReferenceFE(G.lagrangian, float, 1)
    with pytest.raises(NotImplementedError):
        G.TestFESpace(None, reffe, constraint=":zeromean")
