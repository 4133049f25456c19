"""SensorsDict and the uncertainty models on the host (no GPU), with a
stand-in solver whose radiance of a ray is a known function of its
geometry (at3d/containers.py:39-672, at3d/uncertainties.py)."""
import copy

import numpy as np
import pytest

from at3d_gb300.containers import SensorsDict, SolversDict
from at3d_gb300.sensor import make_sensor_dataset, orthographic_projection, stochastic
from at3d_gb300.uncertainties import NullUncertainty, RadiometricUncertainty, TabulatedRadiometricUncertainty
from types import SimpleNamespace


class FakeSolver:
    def __init__(self, scale):
        self.scale = scale
        self.solved = 0
        self.renders = 0

    def check_solved(self, verbose=False):
        return self.solved > 0

    def solve(self, **kw):
        self.solved += 1

    def integrate_to_sensor(self, sensor):
        self.renders += 1
        sensor["I"] = self.scale * (1.0 + np.asarray(sensor["ray_x"]) + 2 * np.asarray(sensor["ray_y"]))
        return sensor


def box():
    return SimpleNamespace(x=np.array([0.0, 1.0]), y=np.array([0.0, 0.5]), z=np.array([0.0, 1.0]))


def make():
    solvers = SolversDict()
    solvers[0.66] = FakeSolver(1.0)
    solvers[0.86] = FakeSolver(2.0)
    sd = SensorsDict()
    sd.add_sensor("cam", orthographic_projection(0.66, box(), 0.1, 0.1, 0.0, 0.0))
    sd.add_sensor("cam", orthographic_projection(0.86, box(), 0.1, 0.1, 30.0, 20.0))
    sub = orthographic_projection(0.66, box(), 0.25, 0.25, 0.0, 0.0,
                                  sub_pixel_ray_args={"method": stochastic, "nrays": 5})
    sd.add_sensor("sub", sub)
    return solvers, sd


def test_get_measurements_splits_rays_back_to_sensors():
    solvers, sd = make()
    sd.get_measurements(solvers)
    assert solvers[0.66].renders == 1 and solvers[0.86].renders == 1    # one render per solver
    for inst in ("cam",):
        for s in sd[inst]["sensor_list"]:
            scale = 1.0 if s["wavelength"] == 0.66 else 2.0
            assert np.allclose(s["I"], scale * (1 + s["ray_x"] + 2 * s["ray_y"]))
    s = sd["sub"]["sensor_list"][0]
    ray = 1 + s["ray_x"] + 2 * s["ray_y"]
    want = np.zeros(len(s["cam_mu"]))
    np.add.at(want, s["pixel_index"], ray * s["ray_weight"])
    assert np.allclose(s["I"], want)
    assert sd.npixels == sum(len(x["cam_mu"]) for i in sd.values() for x in i["sensor_list"])
    assert sd.nmeasurements == sd.npixels
    assert list(sd.get_unique_solvers()) == [0.66, 0.86]


def test_images_and_minimum_stokes():
    solvers, sd = make()
    sd.get_measurements(solvers)
    s = sd["cam"]["sensor_list"][0]
    img = sd.get_image("cam", 0)
    nx, ny = s["image_shape"]
    assert img["I"].shape == (nx, ny)
    assert np.allclose(img["x"][:, 0], np.unique(s["cam_x"]))        # x varies along the first axis
    assert np.allclose(img["I"], img["x"] * 0 + (1 + img["x"] + 2 * img["y"]))
    assert len(sd.get_images("cam")) == 2
    pol = SensorsDict()
    pol.add_sensor("p", make_sensor_dataset([0.5], [0.5], [1.0], [1.0], [0.0], stokes=["I", "Q", "U"],
                                            wavelength=0.66))
    pol.add_sensor("i", make_sensor_dataset([0.5], [0.5], [1.0], [1.0], [0.0], stokes=["I"], wavelength=0.86))
    assert pol.get_minimum_stokes() == {0.66: 3, 0.86: 1}


def test_forward_sensors_are_independent_copies():
    solvers, sd = make()
    fwd = sd.make_forward_sensors()
    fwd.get_measurements(solvers)
    assert "I" in fwd["cam"]["sensor_list"][0] and "I" not in sd["cam"]["sensor_list"][0]
    with pytest.raises(KeyError):
        sd.make_forward_sensors(["nope"])
    with pytest.raises(TypeError):
        sd.get_measurements({0.66: FakeSolver(1.0)})


def test_missing_solver_warns():
    solvers, sd = make()
    solvers[1.6] = FakeSolver(1.0)
    with pytest.warns(UserWarning, match="No sensors"):
        sd.get_measurements(solvers)


def test_null_uncertainty():
    solvers, sd = make()
    sd.get_measurements(solvers)
    sd.add_uncertainty_model("cam", NullUncertainty("L2", 2.0))
    sd.calculate_uncertainties("cam")
    u = sd["cam"]["sensor_list"][0]["uncertainties"]
    assert u.shape == (4, 4, sd["cam"]["sensor_list"][0]["cam_mu"].size) and np.all(u == 2.0)
    assert NullUncertainty("LL").num_uncertainty == 2
    with pytest.raises(ValueError):
        sd.add_noise("cam")
    with pytest.raises(NotImplementedError):
        NullUncertainty("L1")
    with pytest.raises(KeyError):
        sd.calculate_uncertainties("sub")


def test_radiometric_uncertainty():
    s = make_sensor_dataset(np.zeros(20000), np.zeros(20000), np.ones(20000), np.ones(20000), np.zeros(20000),
                            wavelength=0.66)
    s["I"] = np.full(20000, 0.2)
    m = RadiometricUncertainty("L2", lambda r: 100 * np.sqrt(r / 0.2), 1e-4, seed=3)
    m.calculate_uncertainties(s)
    sigma = 0.2 / 100
    assert np.allclose(s["uncertainties"][0, 0], 1 / sigma ** 2)
    assert np.all(s["uncertainties"][1:, 1:] == 1.0)
    noisy = copy.deepcopy(s)
    m.add_noise(noisy)
    # I = sigma sqrt(N), N ~ Poisson((I/sigma)^2): the square root of Poisson counts has a spread of
    # one half, so the perturbation's standard deviation is sigma / 2 (the reference's model)
    assert abs(np.std(noisy["I"]) / (0.5 * sigma) - 1) < 0.05 and abs(np.mean(noisy["I"]) / 0.2 - 1) < 1e-3
    cal = RadiometricUncertainty("L2", lambda r: 100 * np.sqrt(r / 0.2), 1e-4, absolute_calibration_uncertainty=0.03,
                                 camera_to_camera_calibration_uncertainty=0.01, seed=3)
    cal.calculate_uncertainties(s)
    var = sigma ** 2 + (0.01 * 0.2) ** 2 + (cal._absolute_calibration_perturbation * 0.2) ** 2
    assert np.allclose(s["uncertainties"][0, 0], 1 / var)
    tab = TabulatedRadiometricUncertainty("L2", np.array([0.01, 0.05, 0.1, 0.5]), np.array([80.0, 190.0, 270.0, 600.0]))
    snr = tab.noise_curve(np.array([0.001, 0.05, 0.3, 2.0]))
    assert snr[0] == pytest.approx(0.001 / (0.01 / 80.0)) and snr[1] == pytest.approx(190.0)
    assert 270.0 < snr[2] < 600.0 and snr[3] > 600.0


def test_objective_reads_sensors_dict():
    """The retrieval objective takes a SensorsDict: uncertainties per pixel
    and the cost function reach the gradient call, instruments without a
    model get the null model of that cost function, the forward pixel values
    land in forward_sensors, and cost and gradient are per measurement."""
    from at3d_gb300 import gradient, optimize
    seen = []

    def fake_grad(solver, sensor, species=0, **kw):
        seen.append(kw)
        return np.ones((2, 2, 2, 2)), 1.0, np.full(len(sensor["cam_mu"]), 7.0), None

    solvers, sd = make()
    sd.get_measurements(solvers)
    sd.add_uncertainty_model("cam", NullUncertainty("LL", 3.0))
    fwd = sd.make_forward_sensors()
    orig = gradient.levis_approximation_grad
    gradient.levis_approximation_grad = fake_grad
    try:
        with pytest.warns(UserWarning, match="No uncertainty model"):
            obj = optimize.ObjectiveFunction.LevisApproxUncorrelatedL2(
                sd, solvers, fwd, 0, lambda s: None, lambda s, g: sum(v.sum() for v in g.values()) * np.ones(1),
                gradient_kwargs={"cost_function": "LL"})
        loss, grad = obj(np.zeros(1))
    finally:
        gradient.levis_approximation_grad = orig
    n = sd.nmeasurements
    assert loss == pytest.approx(3.0 / n) and grad[0] == pytest.approx(3 * 16.0 / n)
    assert len(seen) == 3 and all(k["cost_function"] == "LL" for k in seen)
    assert seen[0]["uncertainties"].shape[1:] == (2, 2) and np.all(seen[0]["uncertainties"] == 3.0)
    assert np.all(fwd["cam"]["sensor_list"][1]["I"] == 7.0)
    with pytest.raises(ValueError, match="inconsistent"):
        optimize.ObjectiveFunction.LevisApproxUncorrelatedL2(sd, solvers, None, 0, lambda s: None, lambda s, g: 0,
                                                             gradient_kwargs={"cost_function": "L2"})
