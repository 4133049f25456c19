"""The retrieval loop on the host (no GPU): ObjectiveFunction, Optimizer and
the state generators, driven by a stand-in solver whose radiances are a
linear function of extinction (render = A ext, Levis adjoint = A^T w), so the
cost and gradient are known exactly (at3d/optimize.py:20-248)."""
import numpy as np
import pytest

from at3d_gb300.optimize import DensityState, ExtinctionState, ObjectiveFunction, Optimizer


class LinearSolver:
    """Radiance of ray r = sum_i A[r, i] ext_i; ssalb has no effect."""

    def __init__(self, A, shape, ext0):
        self.A = A
        self.shape = shape
        self.ext = np.array(ext0, np.float32).reshape(shape)
        self.ssalb = np.full(shape, 0.99, np.float32)
        self.num_stokes = 1
        self.solves = 0

    def species_properties(self, species=0):
        return self.ext.copy(), self.ssalb.copy()

    def update_species(self, species, extinction=None, ssalb=None):
        if extinction is not None:
            self.ext = np.asarray(extinction, np.float32).reshape(self.shape)
        if ssalb is not None:
            self.ssalb = np.asarray(ssalb, np.float32).reshape(self.shape)

    def solve(self, **kw):
        self.solves += 1

    def check_solved(self, verbose=False):
        return False

    def render(self, x, y, z, mu, phi):
        return (self.A @ self.ext.reshape(-1).astype(np.float64)).astype(np.float32)

    def levis_adjoint(self, rays, weights, species=0):
        g = np.zeros(self.shape + (2,))
        g[..., 0] = (self.A.T @ np.asarray(weights, np.float64)).reshape(self.shape)
        return g


from at3d_gb300.containers import SolversDict as Solvers   # filled by item assignment (no RTE type check)


def sensor(nrays, wavelength, meas):
    z = np.zeros(nrays)
    return {"wavelength": wavelength, "ray_x": z, "ray_y": z, "ray_z": z, "ray_mu": np.ones(nrays),
            "ray_phi": z, "cam_mu": np.ones(nrays), "stokes": [True, False, False, False], "I": meas}


def setup(seed=0, shape=(3, 3, 2), nrays=40):
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    truth = rng.uniform(1.0, 5.0, n)
    solvers = Solvers()
    sensors = []
    for wl in (0.66, 0.86):
        A = rng.uniform(0.0, 0.1, (nrays, n))
        solvers[wl] = LinearSolver(A, shape, np.full(n, 2.0))
        sensors.append(sensor(nrays, wl, (A @ truth).astype(np.float32)))
    return truth.reshape(shape), solvers, sensors


def test_extinction_retrieval_recovers_truth():
    truth, solvers, sensors = setup()
    mask = np.ones(truth.shape, bool)
    state = ExtinctionState(solvers, 0, mask)
    obj = ObjectiveFunction.LevisApproxUncorrelatedL2(sensors, solvers, None, 0, state.set_state,
                                                      state.project_gradient_to_state, min_bounds=0.0,
                                                      max_bounds=10.0)
    seen = []
    opt = Optimizer(obj, callback_fn=lambda optimizer: seen.append(optimizer.iteration),
                    options={"maxiter": 200, "ftol": 1e-14, "gtol": 1e-12})
    x0 = state.initial_state()
    loss0, grad0 = obj(x0)
    # the gradient is the exact gradient of the L2 cost of the linear model
    eps = 1e-3
    for k in (0, 7):
        e = np.zeros_like(x0); e[k] = eps
        fd = (obj(x0 + e)[0] - obj(x0 - e)[0]) / (2 * eps)
        assert fd == pytest.approx(grad0[k], rel=1e-3)
    res = opt.minimize(x0)
    assert res.fun < 1e-6 * loss0
    assert np.allclose(res.x, truth.reshape(-1), rtol=5e-3)
    assert seen == list(range(1, len(seen) + 1)) and opt.iteration == len(seen)
    assert obj.ncalls >= len(seen) and solvers[0.66].solves == obj.ncalls


def test_masked_extinction_leaves_other_points():
    truth, solvers, sensors = setup(1)
    mask = np.zeros(truth.shape, bool)
    mask[1] = True
    state = ExtinctionState(solvers, 0, mask)
    state.set_state(np.arange(mask.sum(), dtype=float))
    for s in solvers.values():
        assert np.array_equal(s.ext[1].reshape(-1), np.arange(mask.sum(), dtype=np.float32))
        assert np.all(s.ext[0] == 2.0) and np.all(s.ext[2] == 2.0)
    g = {0.66: np.ones(truth.shape + (2,)), 0.86: 2 * np.ones(truth.shape + (2,))}
    assert np.array_equal(state.project_gradient_to_state(None, g), np.full(mask.sum(), 3.0))


class FakePoly:
    """A one-coordinate poly table: extinction per density linear in reff."""

    def __init__(self, slope):
        from collections import OrderedDict
        self.coords = OrderedDict(reff=np.array([1.0, 10.0, 30.0]))
        self.extinction = (slope * self.coords["reff"]).astype(np.float32)
        self.ssalb = np.array([0.9, 0.95, 0.99], np.float32)
        leg = np.zeros((6, 3, 3), np.float32)
        leg[0, 0] = 1.0
        self.legcoef = leg


def test_density_state_chain_rule():
    truth, solvers, sensors = setup(2)
    shape = truth.shape
    reff = np.linspace(5.0, 20.0, truth.size).reshape(shape)
    polys = {0.66: FakePoly(2.0), 0.86: FakePoly(3.0)}
    mask = np.ones(shape, bool)
    st = DensityState(solvers, 0, mask, {"reff": reff}, polys, density=np.full(shape, 0.3))
    assert np.allclose(st.per_density[0.66], 2.0 * reff, rtol=1e-6)
    st.set_state(np.full(mask.sum(), 0.5))
    assert np.allclose(solvers[0.86].ext, 0.5 * 3.0 * reff, rtol=1e-6)
    alb = np.interp(reff, [1.0, 10.0, 30.0], [0.9, 0.95, 0.99])
    assert np.allclose(solvers[0.66].ssalb, alb, rtol=1e-6)
    g = {k: np.stack([np.ones(shape), np.zeros(shape)], -1) for k in solvers}
    assert np.allclose(st.project_gradient_to_state(None, g), (5.0 * reff).reshape(-1))


def test_density_retrieval_recovers_truth():
    _, solvers, _ = setup(3)
    shape = (3, 3, 2)
    reff = np.linspace(5.0, 20.0, 18).reshape(shape)
    slopes = {0.66: 0.2, 0.86: 0.3}
    polys = {wl: FakePoly(k) for wl, k in slopes.items()}
    dens_true = np.random.default_rng(4).uniform(0.1, 1.0, shape)
    sensors = []
    for wl, s in solvers.items():
        ext = dens_true * slopes[wl] * reff
        sensors.append(sensor(s.A.shape[0], wl, (s.A @ ext.reshape(-1)).astype(np.float32)))
    mask = np.ones(shape, bool)
    st = DensityState(solvers, 0, mask, {"reff": reff}, polys, density=np.full(shape, 0.5))
    obj = ObjectiveFunction.LevisApproxUncorrelatedL2(sensors, solvers, None, 0, st.set_state,
                                                      st.project_gradient_to_state, min_bounds=0.0,
                                                      max_bounds=5.0)
    res = Optimizer(obj, options={"maxiter": 300, "ftol": 1e-15, "gtol": 1e-12}).minimize(st.initial_state())
    assert np.allclose(res.x, dens_true.reshape(-1), rtol=1e-2)


def test_prior_terms_are_added():
    obj = ObjectiveFunction(None, lambda s, m: (float(np.sum(s ** 2)), 2 * s))
    prior = lambda s, it: (float(np.sum((s - 3) ** 2)), 2 * (s - 3))
    opt = Optimizer(obj, prior_fn=prior, method="L-BFGS-B", options={"maxiter": 100})
    res = opt.minimize(np.zeros(4))
    assert np.allclose(res.x, 1.5, atol=1e-5)      # minimum of x^2 + (x-3)^2
    assert obj.bounds == [(None, None)]
    res = Optimizer(obj, method="CG", options={"maxiter": 100}).minimize(np.ones(3))
    assert np.allclose(res.x, 0.0, atol=1e-5)


def test_unknown_wavelength_is_an_error():
    truth, solvers, sensors = setup(5)
    state = ExtinctionState(solvers, 0, np.ones(truth.shape, bool))
    bad = dict(sensors[0], wavelength=1.6)
    obj = ObjectiveFunction.LevisApproxUncorrelatedL2([bad], solvers, None, 0, state.set_state,
                                                      state.project_gradient_to_state)
    with pytest.raises(KeyError, match="1.6"):
        obj(state.initial_state())


def test_callback_records_iterations():
    from at3d_gb300.optimize import CallbackFn
    obj = ObjectiveFunction(None, lambda s, m: (float(np.sum((s - 1.0) ** 2)), 2 * (s - 1.0)))
    cb = CallbackFn(lambda optimizer: {"iteration": optimizer.iteration, "loss": obj.loss})
    slow = CallbackFn(lambda optimizer: {"iteration": optimizer.iteration}, ckpt_period=3600.0)
    res = Optimizer(obj, callback_fn=[cb, slow], options={"maxiter": 50}).minimize(np.zeros(3))
    assert np.allclose(res.x, 1.0, atol=1e-6)
    assert cb.output["iteration"] == list(range(1, len(cb.output["iteration"]) + 1))
    assert cb.output["loss"][-1] <= cb.output["loss"][0]
    assert slow.output == {}
