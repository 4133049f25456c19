"""Cost functions and adjoint weights of the Levis gradient (host logic,
COMPUTE_ADJOINT_WEIGHTS / UPDATE_COSTFUNCTION) against the reference's own
known answers (tests/test_derivatives.py:75-135 of the reference: a pixel
whose Frechet derivative is one for every Stokes component, so the
gradient is the sum of the adjoint weights)."""
import numpy as np
import pytest

from at3d_gb300.gradient import cost_and_adjoint_weights


def test_l2_known_answer():
    st = np.array([[10.0, 10.0, 10.0, 0.0]])
    me = np.full((1, 4), 13.0)
    un = np.full((1, 4, 4), 5.0)
    cost, adj = cost_and_adjoint_weights(st, me, un, "L2")
    assert cost == pytest.approx(1960.0, abs=1e-5)
    assert adj.sum() == pytest.approx(-440.0, abs=1e-5)


def test_ll_known_answer():
    st = np.array([[1.0, 0.5, 0.0]])
    me = np.array([[1.25, 0.25, 0.25]])
    un = np.zeros((1, 2, 2))
    un[0, 0, 0] = (1.0 / 0.03) ** 2
    un[0, 1, 1] = (1.0 / 0.005) ** 2
    cost, adj = cost_and_adjoint_weights(st, me, un, "LL")
    # the reference's known answer comes from UPDATE_COSTFUNCTION, whose log
    # differences are single precision; the adjoint branch's weights
    # (COMPUTE_ADJOINT_WEIGHTS) are double precision: 1e-6 relative
    assert cost == pytest.approx(6519.21, rel=1e-6)
    assert adj.sum() == pytest.approx(45329.43, rel=1e-6)


def test_adjoint_weights_are_cost_derivatives():
    rng = np.random.default_rng(0)
    st = rng.uniform(0.5, 1.5, (20, 1))
    me = rng.uniform(0.5, 1.5, (20, 1))
    un = rng.uniform(0.5, 2.0, (20, 1, 1))
    for cf in ("L2", "LL"):
        c0, adj = cost_and_adjoint_weights(st, me, un, cf)
        for p in (0, 7, 19):
            h = 1e-6
            s2 = st.copy(); s2[p, 0] += h
            c1, _ = cost_and_adjoint_weights(s2, me, un, cf)
            assert (c1 - c0) / h == pytest.approx(adj[p, 0], rel=1e-4)
    with pytest.raises(ValueError):
        cost_and_adjoint_weights(st, me, un, "XX")
    with pytest.raises(ValueError):
        cost_and_adjoint_weights(-st, me, un, "LL")
