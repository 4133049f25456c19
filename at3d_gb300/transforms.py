"""Maps between the optimiser's abstract state vector and physical fields on
the property grid.

Mirrors at3d.transforms (at3d/transforms.py): coordinate transforms of the
state values (:14-354) and maps from the state vector to the grid
(:356-650).  Each coordinate transform has ``__call__`` (abstract ->
physical), ``inverse_transform`` and ``gradient_transform(abstract,
physical_gradient)``, the chain rule; each grid map has ``__call__`` (state
-> gridded field), ``inverse_transform`` (gridded field -> state),
``gradient_transform`` (gridded gradient -> state gradient) and
``inverse_bounds_transform``.

Differences kept on purpose, so that every ``gradient_transform`` is the
derivative of its ``__call__`` (the optimiser's line search needs that):
* ``CoordinateTransformScaling.gradient_transform`` is g / scaling_factor
  (the reference applies the inverse map, offset included, to the gradient);
* ``CoordinateTransformExp.__call__`` returns -scaling log(1 - a), the
  inverse of its ``inverse_transform`` (the reference returns the negative);
* the profile, column and uniform maps give each state element the sum of
  the gradients of the points it sets (the reference returns their mean).
"""
from __future__ import annotations

import warnings

import numpy as np


class CoordinateTransform:
    """The identity: the state is the physical value."""

    def __call__(self, abstract_state):
        return np.asarray(abstract_state, np.float64)

    def inverse_transform(self, physical_state):
        return np.asarray(physical_state, np.float64)

    def gradient_transform(self, abstract_state, physical_gradient):
        return np.asarray(physical_gradient, np.float64)


class CoordinateTransformLog(CoordinateTransform):
    """State = log(physical)."""

    def __call__(self, abstract_state):
        return np.exp(abstract_state)

    def inverse_transform(self, physical_state):
        return np.log(physical_state)

    def gradient_transform(self, abstract_state, physical_gradient):
        return np.asarray(physical_gradient) * np.exp(abstract_state)


class CoordinateTransformScaling(CoordinateTransform):
    """State = (physical - offset) x scaling_factor."""

    def __init__(self, offset, scaling_factor):
        self._offset = offset
        self._scaling_factor = scaling_factor

    def __call__(self, abstract_state):
        return np.asarray(abstract_state) / self._scaling_factor + self._offset

    def inverse_transform(self, physical_state):
        return (np.asarray(physical_state) - self._offset) * self._scaling_factor

    def gradient_transform(self, abstract_state, physical_gradient):
        return np.asarray(physical_gradient) / self._scaling_factor


class CoordinateTransformExp(CoordinateTransform):
    """State a in [0, 1): physical = -scaling log(1 - a)."""

    def __init__(self, scaling):
        self._scaling = scaling

    def __call__(self, abstract_state):
        return -np.log(1.0 - np.asarray(abstract_state)) * self._scaling

    def inverse_transform(self, physical_state):
        return 1.0 - np.exp(-np.asarray(physical_state) / self._scaling)

    def gradient_transform(self, abstract_state, physical_gradient):
        return -self._scaling * np.asarray(physical_gradient) / (np.asarray(abstract_state) - 1.0)


class CoordinateTransformHyperBol(CoordinateTransform):
    """State a in [0, 1): physical = a / ((1 - a) scaling)."""

    def __init__(self, scaling):
        self._scaling = scaling

    def __call__(self, abstract_state):
        a = np.asarray(abstract_state)
        return (a / (1.0 - a)) / self._scaling

    def inverse_transform(self, physical_state):
        p = np.asarray(physical_state)
        return self._scaling * p / (1.0 + self._scaling * p)

    def gradient_transform(self, abstract_state, physical_gradient):
        a = np.asarray(abstract_state)
        return np.asarray(physical_gradient) / (self._scaling * (1.0 - a) ** 2)


class StateToGridMask:
    """One state element per grid point where ``mask`` is true (all points
    when only ``grid_shape`` is given); other points are 0."""

    def __init__(self, grid_shape=None, mask=None):
        if mask is None and grid_shape is None:
            raise ValueError("At least one of `grid_shape` or `mask` arguments must be provided.")
        if mask is None:
            mask = np.ones(grid_shape, bool)
        elif grid_shape is not None and tuple(grid_shape) != np.asarray(mask).shape:
            raise ValueError("Both `grid_shape` and `mask` arguments were provided. The shape of `mask` is not "
                             "consistent with `grid_shape`.")
        self._mask = np.asarray(mask, bool)
        self._grid_shape = self._mask.shape

    @property
    def mask(self):
        return self._mask

    def __call__(self, state):
        g = np.zeros(self._grid_shape)
        g[self._mask] = state
        return g

    def inverse_transform(self, gridded_data):
        return np.asarray(gridded_data, np.float64)[self._mask]

    def gradient_transform(self, gridded_gradient):
        return np.asarray(gridded_gradient, np.float64)[self._mask]

    def inverse_bounds_transform(self, gridded_bounds):
        return np.asarray(gridded_bounds, np.float64)[self._mask]

    def _uniform_bounds(self, gridded_bounds):
        if np.unique(gridded_bounds).size != 1:
            raise NotImplementedError("Inverse Transform for non-uniform bounds for single variable have not yet "
                                      "been implemented.")
        return self.inverse_transform(gridded_bounds)


class StateToGridProfile(StateToGridMask):
    """One state element per z level: the value of every masked point of the
    level (NaN elsewhere)."""

    def __call__(self, state):
        g = np.full(self._grid_shape, np.nan)
        for i in range(self._grid_shape[-1]):
            g[..., i][self._mask[..., i]] = state[i]
        return g

    def inverse_transform(self, gridded_data):
        g = np.where(self._mask, np.asarray(gridded_data, np.float64), np.nan)
        with warnings.catch_warnings():     # levels without masked points give NaN
            warnings.simplefilter("ignore", RuntimeWarning)
            return np.nanmean(g, axis=(0, 1))

    def gradient_transform(self, gridded_gradient):
        return np.where(self._mask, np.asarray(gridded_gradient, np.float64), 0.0).sum(axis=(0, 1))

    def inverse_bounds_transform(self, gridded_bounds):
        return self._uniform_bounds(gridded_bounds)


class StateToGrid2D(StateToGridMask):
    """One state element per (x, y) column: the value of every masked point
    of the column (NaN elsewhere)."""

    def __call__(self, state):
        s = np.asarray(state).reshape(self._grid_shape[:2])
        return np.where(self._mask, s[..., None], np.nan)

    def inverse_transform(self, gridded_data):
        g = np.where(self._mask, np.asarray(gridded_data, np.float64), np.nan)
        with warnings.catch_warnings():     # columns without masked points give NaN
            warnings.simplefilter("ignore", RuntimeWarning)
            return np.nanmean(g, axis=-1).ravel()

    def gradient_transform(self, gridded_gradient):
        return np.where(self._mask, np.asarray(gridded_gradient, np.float64), 0.0).sum(axis=-1).ravel()

    def inverse_bounds_transform(self, gridded_bounds):
        return self._uniform_bounds(gridded_bounds)


class StateToGridUniform(StateToGridMask):
    """One state element: the value of every masked point (NaN elsewhere)."""

    def __call__(self, state):
        g = np.full(self._grid_shape, np.nan)
        g[self._mask] = np.asarray(state).reshape(-1)[0]
        return g

    def inverse_transform(self, gridded_data):
        return np.atleast_1d(np.mean(np.asarray(gridded_data, np.float64)[self._mask]))

    def gradient_transform(self, gridded_gradient):
        return np.atleast_1d(np.sum(np.asarray(gridded_gradient, np.float64)[self._mask]))

    def inverse_bounds_transform(self, gridded_bounds):
        return self._uniform_bounds(gridded_bounds)
