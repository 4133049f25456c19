"""Measurement uncertainty models: the inverse error covariances that weight
the cost of a retrieval, and measurement noise for synthetic observations.

Mirrors at3d.uncertainties (at3d/uncertainties.py): ``Uncertainty``
(:20-107), ``NullUncertainty`` (:109-141), ``RadiometricUncertainty``
(:143-313) and ``TabulatedRadiometricUncertainty`` (:315-378).  A sensor's
uncertainties are stored as ``sensor['uncertainties']`` [n, n, npixels]
(n = 4 for the 'L2' cost, 2 for 'LL'), the reference's layout; the gradient
takes them per pixel.

Differences kept on purpose: random draws come from a
``numpy.random.Generator`` seeded by ``seed`` instead of the global numpy
state, and ``TabulatedRadiometricUncertainty`` passes its calibration
uncertainties on to the radiometric model (the reference's constructor
drops them).
"""
from __future__ import annotations

import numpy as np

COST_FUNCTIONS = ("L2", "LL")


class Uncertainty:
    """Base class: ``calculate_uncertainties(sensor)`` stores the inverse
    error covariance of every pixel; ``add_noise(sensor)`` perturbs the
    sensor's observables."""

    def __init__(self, cost_function: str):
        if cost_function not in COST_FUNCTIONS:
            raise NotImplementedError(f"`cost_function` '{cost_function}' is not supported for this Uncertainty "
                                      f"type. Valid values are '{COST_FUNCTIONS}'")
        self._cost_function = cost_function
        self._num_uncertainty = 4 if cost_function == "L2" else 2

    def calculate_uncertainties(self, sensor: dict):
        sensor["uncertainties"] = self._process_uncertainties(sensor)

    def add_noise(self, sensor: dict):
        perturbed = self._process_noise(sensor)
        for i, (name, on) in enumerate(zip(("I", "Q", "U", "V"), sensor["stokes"])):
            if on:
                if name not in sensor:
                    raise KeyError(f"Stokes component '{name}' is not found in sensor even though it is an "
                                   "observable. Noise perturbations for this observable cannot be generated.")
                sensor[name] = np.asarray(perturbed[i], np.float64)

    def _process_uncertainties(self, sensor):
        raise NotImplementedError

    def _process_noise(self, sensor):
        raise NotImplementedError

    @property
    def cost_function(self):
        return self._cost_function

    @property
    def num_uncertainty(self):
        return self._num_uncertainty

    @property
    def valid_cost_functions(self):
        return COST_FUNCTIONS


class NullUncertainty(Uncertainty):
    """Unweighted least squares: every inverse covariance element is
    ``scaling_factor``.  It cannot generate noise."""

    def __init__(self, cost_function: str, scaling_factor: float = 1.0):
        super().__init__(cost_function)
        self._scaling_factor = scaling_factor

    def _process_uncertainties(self, sensor):
        n = self._num_uncertainty
        return self._scaling_factor * np.ones((n, n, len(sensor["cam_mu"])))

    def add_noise(self, sensor):
        raise ValueError(f"{type(self)} cannot be used to generate measurement noise. Please assign another "
                         "uncertainty model.")


class RadiometricUncertainty(Uncertainty):
    """Radiometric noise of the intensity: noise standard deviation
    max(I / snr_func(I), sigma_floor) drawn as Poisson counts, times a
    per-sensor camera calibration factor N(1, camera_to_camera) and one
    global factor 1 + N(0, absolute) per model.  The inverse covariance of
    I is 1 / (sigma^2 + (camera I)^2 + (absolute_draw I)^2); the other
    elements are 1."""

    def __init__(self, cost_function: str, snr_func, sigma_floor: float, absolute_calibration_uncertainty=0.0,
                 camera_to_camera_calibration_uncertainty=0.0, seed=None):
        super().__init__(cost_function)
        if not callable(snr_func):
            raise TypeError("snr_func must be a callable of reflectance")
        self._minimum_noise = sigma_floor
        self._snr_func = snr_func
        self._camera = camera_to_camera_calibration_uncertainty
        self._absolute = absolute_calibration_uncertainty
        self._rng = np.random.default_rng(seed)
        self._absolute_calibration_perturbation = self._rng.normal(0.0, absolute_calibration_uncertainty)

    def noise_curve(self, reflectance):
        return self._snr_func(np.atleast_1d(reflectance))

    def _noise_levels(self, radiance):
        snr = np.asarray(self.noise_curve(radiance), np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            levels = np.maximum(radiance / snr, self._minimum_noise)
        levels[snr == 0.0] = self._minimum_noise
        return levels

    def _process_noise(self, sensor, camera_cal=True, noise=True, absolute_cal=True):
        radiance = np.array(sensor["I"], np.float64)
        if noise:
            var = self._noise_levels(radiance) ** 2
            samples = self._rng.poisson(radiance ** 2 / var)
            radiance = np.sqrt(samples * var)
        if camera_cal:
            radiance *= self._rng.normal(1.0, self._camera)
        if absolute_cal:
            radiance *= 1.0 + self._absolute_calibration_perturbation
        out = np.zeros((4, radiance.size))
        out[0] = radiance
        for i, name in enumerate(("Q", "U", "V"), start=1):
            if name in sensor:
                out[i] = sensor[name]
        return out

    def _process_uncertainties(self, sensor, camera_cal=True, noise=True, absolute_cal=True):
        radiance = np.asarray(sensor["I"], np.float64)
        errors = []
        if noise:
            errors.append(self._noise_levels(radiance) ** 2)
        if camera_cal:
            errors.append((self._camera * radiance) ** 2)
        if absolute_cal:
            errors.append((self._absolute_calibration_perturbation * radiance) ** 2)
        u = 1.0 / sum(errors) if errors else np.ones(radiance.shape)
        n = self._num_uncertainty
        big = np.ones((n, n, u.size))
        big[0, 0] = u
        return big


class TabulatedRadiometricUncertainty(RadiometricUncertainty):
    """Radiometric model from a table of SNR at reflectance values: a cubic
    spline inside the table, a + b sqrt(r) fitted to the table above it, and
    the lowest entry's noise level (flat) below it, which is also the noise
    floor."""

    def __init__(self, cost_function: str, reflectance_values, SNR_values, absolute_calibration_uncertainty=0.0,
                 camera_to_camera_calibration_uncertainty=0.0, seed=None):
        import scipy.interpolate as si
        import scipy.optimize as so

        r = np.asarray(reflectance_values, np.float64)
        snr = np.asarray(SNR_values, np.float64)
        noise = r / snr
        spline = si.CubicSpline(r, snr, extrapolate=True)
        fit = lambda x, a, b: a + b * np.sqrt(x)
        popt, _ = so.curve_fit(fit, r, snr, p0=[1e-5, 10])

        def snr_func(x):
            x = np.atleast_1d(np.asarray(x, np.float64))
            out = spline(x)
            hi = x > r.max()
            out[hi] = fit(x[hi], *popt)
            lo = x < r.min()
            out[lo] = x[lo] / noise[0]
            return out

        super().__init__(cost_function, snr_func, noise[0], absolute_calibration_uncertainty,
                         camera_to_camera_calibration_uncertainty, seed)
