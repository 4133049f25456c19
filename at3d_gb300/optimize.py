"""The retrieval loop: a cost and its Levis-approximate gradient as a
function of a state vector, minimised with scipy.

Mirrors at3d.optimize (at3d/optimize.py): ``ObjectiveFunction`` (:20-152)
with its ``LevisApproxUncorrelatedL2`` constructor (:67-145), and
``Optimizer`` (:154-248), a wrapper of ``scipy.optimize.minimize`` that
adds prior terms to the cost and gradient, counts iterations and calls the
user's callbacks with the optimizer.

The state vector maps onto the solvers' media through a state generator,
which takes a coordinate transform and a state-to-grid map
(:mod:`at3d_gb300.transforms`; by default the identity and one element per
masked point) and carries the chain rule through both:

* :class:`ExtinctionState` -- the state sets the extinction of one species
  (the same field in every solver, as for a gray medium);
* :class:`DensityState` -- the state sets the condensate density; each
  solver's extinction is density x the extinction per unit density that its
  poly table gives for the fixed microphysics (reff, veff...), through
  :func:`at3d_gb300.medium.table_to_grid`.  The gradient is the sum over
  solvers of dCost/dExtinction x extinction-per-density.

Prior terms (:mod:`at3d_gb300.regularization`) act on a generator's gridded
field and are passed to :class:`Optimizer` as ``prior_fn``.

Only extinction (or density) is retrieved: the Levis adjoint on the device
gives dCost/dExtinction and dCost/dAlbedo, not the derivative through the
phase functions that a retrieval of effective radius needs.
"""
from __future__ import annotations

import time

import numpy as np



class ObjectiveFunction:
    """The data-misfit term: ``loss_fn(state, measurements) -> (loss,
    gradient)``, with optional per-element bounds for the minimiser."""

    def __init__(self, measurements, loss_fn, min_bounds=None, max_bounds=None):
        self.measurements = measurements
        self.loss_fn = loss_fn
        self._bounds = list(zip(np.atleast_1d(min_bounds), np.atleast_1d(max_bounds)))
        self._loss = None
        self._total_obj_fn_time = 0.0
        self._ncalls = 0

    def __call__(self, state):
        t0 = time.perf_counter()
        loss, gradient = self.loss_fn(state, self.measurements)
        self._total_obj_fn_time += time.perf_counter() - t0
        self._loss = loss
        self._ncalls += 1
        return loss, gradient

    @classmethod
    def LevisApproxUncorrelatedL2(cls, measurements, solvers, forward_sensors, unknown_scatterers, set_state_fn,
                                  project_gradient_to_state, parallel_solve_kwargs=None, gradient_kwargs=None,
                                  uncertainty_kwargs=None, min_bounds=None, max_bounds=None):
        """The uncertainty-weighted misfit of the measurements and its
        Levis-approximate gradient (at3d/optimize.py:67-145), through
        :class:`at3d_gb300.gradient.LevisApproxGradientUncorrelated`: each
        call sets the state (``set_state_fn(state)``), solves, and maps the
        gridded gradients onto the state with
        ``project_gradient_to_state(state, {solver key: gradient [npx, npy,
        npz, 2]})``; cost and gradient are divided by the number of
        measurements.  ``measurements``: a SensorsDict (or a list of sensor
        dicts, taken as one instrument with unit uncertainties), each sensor
        with its 'wavelength' (the key of its solver) and measured 'I';
        ``forward_sensors`` (or None) receives the forward model's pixel
        values; ``unknown_scatterers``: the species index whose extinction
        and albedo are differentiated."""
        from .containers import SensorsDict
        from .gradient import LevisApproxGradientUncorrelated
        if not isinstance(measurements, SensorsDict):
            from .uncertainties import NullUncertainty
            sd = SensorsDict()
            cost = (gradient_kwargs or {}).get("cost_function", "L2")
            sd.add_uncertainty_model("sensors", NullUncertainty(cost))
            for sensor in measurements:
                sd.add_sensor("sensors", sensor)
            measurements = sd
        gradient_fn = LevisApproxGradientUncorrelated(measurements, solvers, forward_sensors, unknown_scatterers,
                                                      parallel_solve_kwargs, gradient_kwargs, uncertainty_kwargs)

        def loss_function(state, measurements):
            set_state_fn(state)
            loss, gradient, _ = gradient_fn()
            return loss, project_gradient_to_state(state, gradient)

        return cls(measurements, loss_function, min_bounds=min_bounds, max_bounds=max_bounds)

    @property
    def loss(self):
        return self._loss

    @property
    def bounds(self):
        return self._bounds

    @property
    def ncalls(self):
        return self._ncalls


class Optimizer:
    """scipy.optimize.minimize over an :class:`ObjectiveFunction`, with prior
    terms ``prior(state, iteration) -> (loss, gradient)`` added to the cost
    and callbacks ``callback(optimizer=self)`` after every iteration."""

    def __init__(self, objective_fn, prior_fn=None, callback_fn=None, method="L-BFGS-B",
                 options=None):
        self._method = method
        self._options = dict(options) if options is not None else \
            {"maxiter": 100, "maxls": 10, "disp": False, "gtol": 1e-16, "ftol": 1e-8}
        self._objective_fn = objective_fn
        self._prior_fn = list(np.atleast_1d(prior_fn)) if prior_fn is not None else None
        self._callback_fn = list(np.atleast_1d(callback_fn)) if callback_fn is not None else []
        self._iteration = None
        self._state = None

    def callback(self, state):
        self._iteration += 1
        for fn in self._callback_fn:
            fn(optimizer=self)

    def objective(self, state):
        self._state = state
        loss, gradient = self._objective_fn(state)
        gradient = np.array(gradient, np.float64, copy=True)
        if self._prior_fn is not None:
            for prior in self._prior_fn:
                ploss, pgrad = prior(state, self._iteration)
                loss += ploss
                gradient += pgrad
        return loss, gradient

    def minimize(self, initial_state, iteration_step=0, **kwargs):
        """Local minimisation from ``initial_state``; returns scipy's result."""
        import scipy.optimize

        self._iteration = iteration_step
        args = {"fun": self.objective, "x0": np.asarray(initial_state, np.float64), "method": self._method,
                "jac": True, "options": self._options, "callback": self.callback}
        args.update(kwargs)
        if self._method not in ("CG", "Newton-CG") and "bounds" not in kwargs:
            bounds = self._objective_fn.bounds
            n = len(args["x0"])
            if len(bounds) == 1:
                args["bounds"] = [bounds[0]] * n
            elif len(bounds) == n:
                args["bounds"] = bounds
        return scipy.optimize.minimize(**args)

    @property
    def objective_fn(self):
        return self._objective_fn

    @property
    def iteration(self):
        return self._iteration

    @property
    def method(self):
        return self._method

    @property
    def options(self):
        return self._options

    @property
    def state(self):
        return self._state


class _GridState:
    """A state vector mapped onto one field of the property grid: physical =
    transform(state) placed on the grid by ``state_to_grid`` (default: one
    element per point of ``mask``); the points the map does not set keep
    their current values."""

    def __init__(self, solvers, species: int, mask=None, transform=None, state_to_grid=None, grid=None,
                 grid_shape=None):
        from .transforms import CoordinateTransform, StateToGridMask
        self.solvers = solvers
        self.species = species
        if state_to_grid is None:
            if mask is None and grid_shape is None:
                raise ValueError("give a mask, a grid shape or a state_to_grid map")
            state_to_grid = StateToGridMask(grid_shape=grid_shape, mask=mask)
        self.state_to_grid = state_to_grid
        self.transform = transform if transform is not None else CoordinateTransform()
        self.mask = np.asarray(state_to_grid.mask, bool)
        self._grid = grid

    @property
    def grid_shape(self):
        return self.mask.shape

    @property
    def grid(self):
        """The property grid (x, y, z) of the first solver, for smoothing priors."""
        if self._grid is None:
            from .grid import make_grid
            pb = next(iter(self.solvers.values())).problem
            npx, npy, _ = self.grid_shape
            self._grid = make_grid(pb.delx, npx, pb.dely, npy, pb.zlevels)
        return self._grid

    def gridded(self, state):
        """The physical field the state sets (NaN or 0 where it sets nothing)."""
        return self.state_to_grid(self.transform(np.asarray(state, np.float64)))

    def project_gridded_gradient(self, state, gridded_gradient):
        """d/d(state) from d/d(gridded field), through the map and the transform."""
        return self.transform.gradient_transform(np.asarray(state, np.float64),
                                                 self.state_to_grid.gradient_transform(gridded_gradient))

    def _state_of(self, field):
        return self.transform.inverse_transform(self.state_to_grid.inverse_transform(field))

    def _place(self, current, state):
        out = np.array(current, np.float64, copy=True)
        out[self.mask] = self.gridded(state)[self.mask]
        return out


class ExtinctionState(_GridState):
    """State = the extinction of ``species`` where the map sets it (by default
    one element per point of ``mask``), the same in every solver."""

    def initial_state(self, key=None):
        s = self.solvers[key if key is not None else next(iter(self.solvers))]
        ext, _ = s.species_properties(self.species)
        return self._state_of(np.asarray(ext, np.float64))

    def set_state(self, state):
        for solver in self.solvers.values():
            ext, _ = solver.species_properties(self.species)
            solver.update_species(self.species, extinction=self._place(ext, state).astype(np.float32))

    def project_gradient_to_state(self, state, gradients):
        total = sum(np.asarray(g[..., 0], np.float64) for g in gradients.values())
        return self.project_gridded_gradient(state, total)


class DensityState(_GridState):
    """State = the condensate density where the map sets it.  ``microphysics``:
    the fixed parameters of the table (e.g. {'reff': [...], 'veff': [...]},
    arrays on the property grid); ``poly_tables``: {solver key: PolyTable}.
    The phase functions stay as the solvers hold them (density does not
    change them); the albedo is set from the table."""

    def __init__(self, solvers, species: int, mask, microphysics: dict, poly_tables: dict, density=None,
                 transform=None, state_to_grid=None, grid=None):
        from .medium import table_to_grid
        super().__init__(solvers, species, mask, transform, state_to_grid, grid)
        shape = self.mask.shape
        self.density = np.zeros(shape) if density is None else np.array(density, np.float64, copy=True)
        self.per_density = {}
        self.ssalb = {}
        for key in solvers:
            sp = table_to_grid(dict(microphysics, density=np.ones(shape)), poly_tables[key], inverse_mode=True)
            self.per_density[key] = np.asarray(sp.extinction, np.float64)
            self.ssalb[key] = np.asarray(sp.ssalb, np.float32)

    def initial_state(self):
        return self._state_of(self.density)

    def set_state(self, state):
        self.density = self._place(self.density, state)
        for key, solver in self.solvers.items():
            ext = (self.density * self.per_density[key]).astype(np.float32)
            solver.update_species(self.species, extinction=ext, ssalb=self.ssalb[key])

    def project_gradient_to_state(self, state, gradients):
        total = sum(np.asarray(g[..., 0], np.float64) * self.per_density[k] for k, g in gradients.items())
        return self.project_gridded_gradient(state, total)


class CallbackFn:
    """An Optimizer callback that records what ``callback_fn(optimizer=...)``
    returns (a dict of values) at most once every ``ckpt_period`` seconds
    (every iteration with the default of -1) into ``self.output`` {name:
    [value per recorded iteration]} (at3d/callback.py:32-49).  The
    reference's tensorboard writer is not included."""

    def __init__(self, callback_fn, ckpt_period=-1):
        self._ckpt_period = ckpt_period
        self._ckpt_time = time.time()
        self._callback_fn = callback_fn
        self.output = {}

    def __call__(self, optimizer=None):
        if time.time() - self._ckpt_time > self._ckpt_period:
            self._ckpt_time = time.time()
            out = self._callback_fn(optimizer=optimizer)
            for name, value in out.items():
                self.output.setdefault(name, []).append(value)
