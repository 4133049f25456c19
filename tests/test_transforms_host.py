"""State transforms and priors of the retrieval loop on the host (no GPU):
every gradient_transform is the derivative of its map, grid_smoothing's
gradient is the derivative of its cost (src/util.f90:65-238), and a
log-state retrieval with a smoothing prior runs through Optimizer
(at3d/transforms.py, at3d/regularization.py)."""
import numpy as np
import pytest

from at3d_gb300 import regularization as R
from at3d_gb300 import transforms as T


@pytest.mark.parametrize("tr, a", [
    (T.CoordinateTransform(), np.array([0.3, 2.0, 5.0])),
    (T.CoordinateTransformLog(), np.array([-1.0, 0.2, 1.5])),
    (T.CoordinateTransformScaling(2.0, 5.0), np.array([-1.0, 0.2, 1.5])),
    (T.CoordinateTransformExp(3.0), np.array([0.1, 0.5, 0.9])),
    (T.CoordinateTransformHyperBol(2.0), np.array([0.1, 0.5, 0.9])),
])
def test_coordinate_transforms(tr, a):
    assert np.allclose(tr.inverse_transform(tr(a)), a)
    g = np.array([0.7, -1.3, 2.1])
    h = 1e-6
    fd = (tr(a + h) - tr(a - h)) / (2 * h) * g          # d/da of sum g p(a)
    assert np.allclose(tr.gradient_transform(a, g), fd, rtol=1e-5)


@pytest.mark.parametrize("cls", [T.StateToGridMask, T.StateToGridProfile, T.StateToGrid2D, T.StateToGridUniform])
def test_grid_maps_are_adjoint(cls):
    rng = np.random.default_rng(0)
    mask = rng.uniform(size=(4, 3, 5)) > 0.4
    m = cls(mask=mask)
    n = {T.StateToGridMask: mask.sum(), T.StateToGridProfile: 5, T.StateToGrid2D: 12, T.StateToGridUniform: 1}[cls]
    s = rng.uniform(1, 2, n)
    field = m(s)
    assert np.all(np.isfinite(field[mask]))
    g = rng.normal(size=mask.shape)
    # sum_masked g * map(s) is linear in s: its gradient is gradient_transform(g)
    lin = lambda st: float(np.sum(np.where(mask, g * np.nan_to_num(m(st)), 0.0)))
    e = np.eye(n)
    num = np.array([lin(e[i]) for i in range(n)])
    assert np.allclose(m.gradient_transform(np.where(mask, g, 0.0)), num)
    if cls is not T.StateToGridMask:
        back = m.inverse_transform(field)
        ok = np.isfinite(back)
        assert np.allclose(back[ok], np.asarray(s).reshape(-1)[ok])
    assert np.array_equal(T.StateToGridMask(grid_shape=(2, 2, 2)).mask, np.ones((2, 2, 2), bool))
    with pytest.raises(ValueError):
        T.StateToGridMask()


@pytest.mark.parametrize("mode", ["l2", "ph", "l1"])
def test_grid_smoothing_gradient(mode):
    rng = np.random.default_rng(1)
    x, y, z = np.cumsum(rng.uniform(0.5, 1.5, 4)), np.cumsum(rng.uniform(0.5, 1.5, 5)), np.cumsum(rng.uniform(0.5, 1.5, 3))
    f = rng.normal(size=(4, 5, 3))
    w = rng.uniform(0.5, 1.5, size=f.shape)
    cost, grad = R.grid_smoothing(f, w, x, y, z, mode=mode, direction_weights=(1.0, 0.5, 2.0), huber_parameter=0.7)
    assert cost > 0
    if mode == "l1":
        # the subgradient of the edge signs: a small step along -grad lowers the cost
        c2, _ = R.grid_smoothing(f - 1e-4 * grad, w, x, y, z, mode=mode, direction_weights=(1.0, 0.5, 2.0))
        assert c2 < cost
        return
    h = 1e-6
    num = np.zeros_like(f)
    for idx in np.ndindex(f.shape):
        e = np.zeros_like(f); e[idx] = h
        num[idx] = (R.grid_smoothing(f + e, w, x, y, z, mode=mode, direction_weights=(1.0, 0.5, 2.0),
                                     huber_parameter=0.7)[0] -
                    R.grid_smoothing(f - e, w, x, y, z, mode=mode, direction_weights=(1.0, 0.5, 2.0),
                                     huber_parameter=0.7)[0]) / (2 * h)
    assert np.allclose(grad, num, rtol=1e-5, atol=1e-8)
    # a constant field has no cost
    assert R.grid_smoothing(np.ones_like(f), w, x, y, z, mode=mode)[0] == pytest.approx(0.0, abs=1e-12)


def test_log_state_retrieval_with_priors():
    from test_optimize_host import setup
    from at3d_gb300.grid import make_grid
    from at3d_gb300.optimize import ExtinctionState, ObjectiveFunction, Optimizer
    truth, solvers, sensors = setup(7)
    state = ExtinctionState(solvers, 0, np.ones(truth.shape, bool), transform=T.CoordinateTransformLog(),
                            grid=make_grid(0.1, 3, 0.1, 3, [0.0, 0.1]))
    obj = ObjectiveFunction.LevisApproxUncorrelatedL2(sensors, solvers, None, 0, state.set_state,
                                                      state.project_gradient_to_state)
    smooth = R.SpatialSmoothing(state, 1e-6, mode="l2")
    tik = R.Tikhonov(state, 1e-7)
    opt = Optimizer(obj, prior_fn=[smooth, tik], options={"maxiter": 300, "ftol": 1e-15, "gtol": 1e-12})
    x0 = state.initial_state()
    assert np.allclose(np.exp(x0), 2.0)
    # the whole objective's gradient (data term and priors, through the log state) against differences
    # (the stand-in solver keeps extinction in single precision, hence the step of 1e-3)
    f0, g0 = opt.objective(x0)
    for k in (0, 5, 11):
        e = np.zeros_like(x0); e[k] = 1e-3
        fd = (opt.objective(x0 + e)[0] - opt.objective(x0 - e)[0]) / 2e-3
        assert fd == pytest.approx(g0[k], rel=1e-3)
    res = opt.minimize(x0)
    assert np.allclose(np.exp(res.x), truth.reshape(-1), rtol=2e-2)
    cost, grad = R.PriorCovariance(np.eye(3) * 2.0, np.ones(3))(np.array([1.0, 2.0, 0.0]))
    assert cost == pytest.approx(4.0) and np.allclose(grad, [0.0, 4.0, -4.0])
    with pytest.raises(ValueError):
        R.Tikhonov(state, -1.0)
    with pytest.raises(ValueError):
        R.SpatialSmoothing(state, 1.0, mode="l3")
