"""Prior terms of the retrieval cost, as ``prior(state, iteration) ->
(cost, gradient with respect to the state)`` for ``optimize.Optimizer``.

Mirrors at3d.regularization (at3d/regularization.py): ``Sparsity``
(:202-249), ``Tikhonov`` (:251-300), ``SpatialSmoothing`` (:311-388, the
cost and gradient of GRID_SMOOTHING, src/util.f90:65-238) and
``PriorCovariance`` (:390-403).  A term acts on the gridded physical field
of a state generator (``optimize.ExtinctionState``, ``DensityState``:
``gridded(state)`` and ``project_gridded_gradient(state, gradient)``) and is
scaled by strength x relaxation^iteration.

Differences kept on purpose: ``Sparsity`` and ``Tikhonov`` weight each
point by ``spatial_weights`` (the reference stores the weights but does not
use them; with the default weights of one the results agree), and the
``direction_weights`` of ``SpatialSmoothing`` are ordered (x, y, z) (the
reference's call applies its first weight along z).
"""
from __future__ import annotations

import numpy as np


class Regularization:
    def __init__(self, state_generator, regularization_strength: float, relaxation_parameter: float = 1.0):
        if not isinstance(regularization_strength, float) or regularization_strength < 0.0:
            raise ValueError("`regularization_strength` should be a positive float.")
        if not isinstance(relaxation_parameter, float) or relaxation_parameter < 0.0:
            raise ValueError("`relaxation_parameter` should be a positive float.")
        for m in ("gridded", "project_gridded_gradient"):
            if not hasattr(state_generator, m):
                raise TypeError(f"`state_generator` needs a '{m}' method")
        self._state_generator = state_generator
        self._regularization_strength = regularization_strength
        self._relaxation_parameter = relaxation_parameter

    @property
    def state_generator(self):
        return self._state_generator

    def regularization_strength(self, iteration_number) -> float:
        return self._regularization_strength * self._relaxation_parameter ** (iteration_number or 0)

    def _field(self, state):
        """The generator's physical field on the grid (0 where the state does not reach)."""
        g = np.asarray(self._state_generator.gridded(state), np.float64)
        return np.where(np.isnan(g), 0.0, g)


class WeightedRegularization(Regularization):
    def __init__(self, state_generator, regularization_strength, relaxation_parameter=1.0, spatial_weights=None):
        super().__init__(state_generator, regularization_strength, relaxation_parameter)
        shape = state_generator.grid_shape
        if spatial_weights is None:
            spatial_weights = np.ones(shape)
        if not isinstance(spatial_weights, np.ndarray):
            raise TypeError("`spatial_weights` should be a numpy array.")
        if spatial_weights.shape != tuple(shape):
            raise ValueError("`spatial_weights` should be of the same shape as the property grid.")
        if np.any(spatial_weights < 0.0):
            raise ValueError("`spatial_weights` should be positive floats.")
        self._spatial_weights = spatial_weights


class Sparsity(WeightedRegularization):
    """strength x sum w |f|."""

    def __call__(self, state, iteration_number):
        f, s = self._field(state), self.regularization_strength(iteration_number)
        cost = s * float(np.sum(self._spatial_weights * np.abs(f)))
        return cost, self._state_generator.project_gridded_gradient(state, s * self._spatial_weights * np.sign(f))


class Tikhonov(WeightedRegularization):
    """strength x sum w f^2."""

    def __call__(self, state, iteration_number):
        f, s = self._field(state), self.regularization_strength(iteration_number)
        cost = s * float(np.sum(self._spatial_weights * f * f))
        return cost, self._state_generator.project_gridded_gradient(state, s * 2.0 * self._spatial_weights * f)


def grid_smoothing(field, weights, xgrid, ygrid, zgrid, mode="l2", direction_weights=(1.0, 1.0, 1.0),
                   huber_parameter=1.0):
    """GRID_SMOOTHING (src/util.f90:65-238) on fields [nx, ny, nz]: per grid
    cell, the cell-averaged derivatives along x, y, z (the mean of the four
    edge differences along each axis over the spacing) and the cell volume
    times the mean weight of its corners; cost = sum of volume x ('l2') the
    direction-weighted squared derivatives, ('l1') the weighted absolute
    derivatives, ('ph') the pseudo-Huber h^2 (sqrt(1 + n/h^2) - 1) of the
    squared norm n.  The gradient is the cost's derivative ('l1': each edge
    contributes its own sign, as there).  Returns (cost, gradient)."""
    if mode not in ("l1", "l2", "ph"):
        raise ValueError(f"GRID_SMOOTHING: Unrecognized argument for 'mode' {mode}")
    F = np.asarray(field, np.float64)
    W = np.asarray(weights, np.float64)
    wx, wy, wz = (float(v) for v in direction_weights)
    dx = np.diff(np.asarray(xgrid, np.float64))[:, None, None]
    dy = np.diff(np.asarray(ygrid, np.float64))[None, :, None]
    dz = np.diff(np.asarray(zgrid, np.float64))[None, None, :]
    c = lambda A, i, j, k: A[i:A.shape[0] - 1 + i, j:A.shape[1] - 1 + j, k:A.shape[2] - 1 + k]
    vol = dx * dy * dz * 0.125 * sum(c(W, i, j, k) for i in (0, 1) for j in (0, 1) for k in (0, 1))
    ex = [c(F, 1, j, k) - c(F, 0, j, k) for j in (0, 1) for k in (0, 1)]     # edges along x
    ey = [c(F, i, 1, k) - c(F, i, 0, k) for i in (0, 1) for k in (0, 1)]
    ez = [c(F, i, j, 1) - c(F, i, j, 0) for i in (0, 1) for j in (0, 1)]
    xd, yd, zd = 0.25 * sum(ex) / dx, 0.25 * sum(ey) / dy, 0.25 * sum(ez) / dz
    grad = np.zeros_like(F)

    def add(i, j, k, v):
        grad[i:F.shape[0] - 1 + i, j:F.shape[1] - 1 + j, k:F.shape[2] - 1 + k] += v

    if mode == "l1":
        cost = float(np.sum(vol * (wx * np.abs(xd) + wy * np.abs(yd) + wz * np.abs(zd))))
        sgn = lambda e, w: np.where(e >= 0.0, w, -w)        # Fortran SIGN(w, e): +w for e = 0
        for n, (j, k) in enumerate((j, k) for j in (0, 1) for k in (0, 1)):
            v = vol * sgn(ex[n], wx) / dx
            add(0, j, k, -v); add(1, j, k, v)
        for n, (i, k) in enumerate((i, k) for i in (0, 1) for k in (0, 1)):
            v = vol * sgn(ey[n], wy) / dy
            add(i, 0, k, -v); add(i, 1, k, v)
        for n, (i, j) in enumerate((i, j) for i in (0, 1) for j in (0, 1)):
            v = vol * sgn(ez[n], wz) / dz
            add(i, j, 0, -v); add(i, j, 1, v)
        return cost, 0.25 * grad
    norm = wx * xd * xd + wy * yd * yd + wz * zd * zd
    if mode == "l2":
        cost, scale = float(np.sum(vol * norm)), vol
    else:
        h2 = huber_parameter ** 2
        cost = float(np.sum(vol * h2 * (np.sqrt(1.0 + norm / h2) - 1.0)))
        scale = vol / np.sqrt(1.0 + norm / h2)
    for i in (0, 1):
        for j in (0, 1):
            for k in (0, 1):
                s = lambda b: 1.0 if b else -1.0
                add(i, j, k, scale * (s(i) * wx * xd / dx + s(j) * wy * yd / dy + s(k) * wz * zd / dz))
    grad *= 0.25
    if mode == "l2":
        grad *= 2.0
    return cost, grad


class SpatialSmoothing(WeightedRegularization):
    """strength x GRID_SMOOTHING of the field (modes 'l1', 'l2', 'ph')."""

    def __init__(self, state_generator, regularization_strength, relaxation_parameter=1.0, mode="l2",
                 direction_weights=(1.0, 1.0, 1.0), spatial_weights=None, huber_parameter=1.0, grid=None):
        super().__init__(state_generator, regularization_strength, relaxation_parameter, spatial_weights)
        if mode not in ("l1", "l2", "ph"):
            raise ValueError(f"Spatial Smoothing `mode` should be in {('l1', 'l2', 'ph')}")
        self._mode = mode
        self._direction_weights = np.atleast_1d(direction_weights)
        self._huber_parameter = huber_parameter
        g = grid if grid is not None else state_generator.grid
        self._coords = (np.asarray(g.x), np.asarray(g.y), np.asarray(g.z))

    def __call__(self, state, iteration_number):
        f, s = self._field(state), self.regularization_strength(iteration_number)
        cost, grad = grid_smoothing(f, self._spatial_weights, *self._coords, mode=self._mode,
                                    direction_weights=self._direction_weights, huber_parameter=self._huber_parameter)
        return s * cost, self._state_generator.project_gridded_gradient(state, s * grad)


class PriorCovariance:
    """Gaussian prior on the state: (x - c)^T C^-1 (x - c) and its gradient."""

    def __init__(self, inverse_covariance, central_vector):
        self._inverse_covariance = np.asarray(inverse_covariance, np.float64)
        self._central_vector = np.asarray(central_vector, np.float64)

    def __call__(self, state, iteration_number=None):
        d = np.asarray(state, np.float64) - self._central_vector
        g = self._inverse_covariance @ d
        return float(d @ g), 2.0 * g
