"""Sensors: the pixel and ray geometry that ``RTE.integrate_to_sensor``
renders, and the pixel averages of the rendered rays.

Mirrors the sensor-generating calls of ``at3d.sensor`` (at3d/sensor.py):
``make_sensor_dataset`` (:31-106), the sub-pixel ray samplers
``stochastic``, ``uniform`` and ``gaussian`` (:109-186),
``orthographic_projection`` (:188-347), ``perspective_projection``
(:367-553) and ``domaintop_projection`` (:555-622), with the same
arguments, conventions and ray layout.  A sensor is a plain dict instead
of an ``xr.Dataset`` (xarray is not a dependency here): pixel variables
``cam_x/y/z/mu/phi`` over the pixels, ray variables ``ray_x/y/z/mu/phi``,
``pixel_index`` and ``ray_weight`` over the rays, ``image_shape`` and the
projection's attributes.  mu and phi point from the scene TOWARDS the
sensor (at3d/sensor.py:44-47).

``calculate_observables`` is SensorsDict._calculate_observables
(at3d/containers.py:600-650): pixel Stokes values as ray-weighted sums of
the rendered rays (``average_subpixel_rays``, src/util.f90:484-519).
"""
from __future__ import annotations

import inspect
import itertools

import numpy as np

STOKES_NAMES = ("I", "Q", "U", "V")


def make_sensor_dataset(x, y, z, mu, phi, stokes=("I",), wavelength=None, fill_ray_variables=True) -> dict:
    """Pixel geometry of a sensor (at3d/sensor.py:31-106); with
    ``fill_ray_variables`` one ray per pixel (the reference's default when
    no projection generates sub-pixel rays is False; here True, since a
    sensor without rays cannot be rendered)."""
    x, y, z, mu, phi = (np.asarray(v) for v in (x, y, z, mu, phi))
    stokes = [str(s) for s in np.atleast_1d(stokes)]
    for v, name in zip((x, y, z, mu, phi), ("x", "y", "z", "mu", "phi")):
        if v.ndim != 1:
            raise ValueError(f"'{name}' should be a 1-D np.ndarray")
    if not all(x.size == v.size for v in (y, z, mu, phi)):
        raise ValueError("All of x, y, z, mu, phi should have the same size.")
    if not np.all(z >= 0.0):
        raise ValueError("All altitudes (z) must be >= 0.0")
    if np.any(mu == 0.0):
        raise ValueError("'mu' values of 0.0 are not allowed.")
    for s in stokes:
        if s not in STOKES_NAMES:
            raise ValueError(f"Valid Stokes components are 'I', 'Q', 'U', 'V' not '{s}'")
    sensor = {"wavelength": wavelength, "stokes": [s in stokes for s in STOKES_NAMES],
              "cam_x": x.astype(np.float64), "cam_y": y.astype(np.float64), "cam_z": z.astype(np.float64),
              "cam_mu": mu.astype(np.float64), "cam_phi": phi.astype(np.float64), "attrs": {}}
    if fill_ray_variables:
        _add_null_subpixel_rays(sensor)
    return sensor


def _add_null_subpixel_rays(sensor: dict) -> dict:
    """One ray per pixel (at3d/sensor.py:661-681)."""
    for name in ("x", "y", "z", "mu", "phi"):
        sensor["ray_" + name] = np.array(sensor["cam_" + name], np.float64)
    n = len(sensor["cam_mu"])
    sensor["pixel_index"] = np.arange(n)
    sensor["ray_weight"] = np.ones(n)
    sensor["use_subpixel_rays"] = False
    return sensor


def stochastic(npixels, nrays, seed=None):
    """Uniform random position perturbations in (-1, 1] and equal weights
    1/nrays per pixel (at3d/sensor.py:109-141)."""
    rng = np.random.RandomState(seed) if seed is not None else np.random
    pert = rng.uniform(low=-1.0, high=1.0, size=(npixels, nrays))
    return pert, np.ones((npixels, nrays)) / nrays


def uniform(npixels, nrays):
    """nrays evenly spaced perturbations, equal weights (at3d/sensor.py:143-146)."""
    pert = np.linspace(-1.0 + 1 / nrays, 1.0 - 1 / nrays, nrays)
    return pert, np.ones((npixels, nrays)) / nrays


def gaussian(npixels, degree):
    """Gauss-Legendre positions and weights (normalised to sum to one) of
    the given degree (at3d/sensor.py:148-186)."""
    x, w = np.polynomial.legendre.leggauss(degree)
    return np.repeat(x[np.newaxis, :], npixels, axis=0), np.repeat(w[np.newaxis, :], npixels, axis=0) / np.sum(w)


def _parse_sub_pixel_ray_args(args: dict):
    """Split a sub_pixel_ray_args dict into the method and its keyword
    arguments for the image x and y axes (a tuple value gives (x, y))."""
    method = args.get("method")
    if not callable(method):
        raise TypeError(f"sub_pixel_ray_args 'method' must be a callable object not '{method}'")
    params = inspect.signature(method).parameters
    kx, ky = {}, {}
    for name, value in args.items():
        if name == "method":
            continue
        if name not in params:
            raise KeyError(f"Invalid kwarg '{name}' passed to the sub_pixel_ray_args method '{method.__name__}'")
        if isinstance(value, tuple):
            kx[name], ky[name] = value
        else:
            kx[name] = ky[name] = value
    return method, kx, ky


def orthographic_projection(wavelength, bounding_box, x_resolution, y_resolution, azimuth, zenith,
                            altitude="TOA", stokes="I", sub_pixel_ray_args=None) -> dict:
    """Parallel rays viewing the bounding box (anything with x, y, z
    coordinate arrays, e.g. a ``grid.Grid``) at one zenith / azimuth
    (degrees, photon direction) with pixel spacing x_resolution,
    y_resolution on the horizontal (at3d/sensor.py:188-347): the box's
    eight corners are projected along the view onto the altitude plane and
    the pixels cover that footprint, padded to include its far edge."""
    sub_pixel_ray_args = dict(sub_pixel_ray_args or {"method": None})
    mu = np.cos(np.deg2rad(zenith))
    phi = np.deg2rad(azimuth)
    bx, by, bz = (np.asarray(getattr(bounding_box, k)) for k in ("x", "y", "z"))
    xmin, ymin, zmin = bx.min(), by.min(), bz.min()
    xmax, ymax, zmax = bx.max(), by.max(), bz.max()
    altitude = zmax if altitude == "TOA" else altitude
    alpha = np.sqrt(1 - mu ** 2) * np.cos(phi) / mu
    beta = np.sqrt(1 - mu ** 2) * np.sin(phi) / mu
    proj = np.array([[1, 0, -alpha, alpha * altitude], [0, 1, -beta, beta * altitude], [0, 0, 0, altitude]])
    corners = np.array(list(itertools.product([xmin, xmax], [ymin, ymax], [zmin, zmax]))).T
    fp = proj @ np.pad(corners, ((0, 1), (0, 0)), "constant", constant_values=1)
    x_s, y_s = fp[:2].min(axis=1)
    x_e, y_e = fp[:2].max(axis=1)
    x = np.arange(x_s, x_e + x_resolution, x_resolution)
    y = np.arange(y_s, y_e + y_resolution, y_resolution)
    image_shape = [x.size, y.size]
    X, Y, Z, MU, PHI = np.meshgrid(x, y, altitude, mu, phi)
    sensor = make_sensor_dataset(X.ravel(), Y.ravel(), Z.ravel(), MU.ravel(), PHI.ravel(), stokes, wavelength,
                                 fill_ray_variables=False)
    sensor["bounding_box"] = np.array([xmin, ymin, zmin, xmax, ymax, zmax])
    sensor["image_shape"] = image_shape
    sensor["attrs"] = {"projection": "Orthographic", "altitude": altitude, "x_resolution": x_resolution,
                       "y_resolution": y_resolution, "projection_azimuth": azimuth, "projection_zenith": zenith}
    if sub_pixel_ray_args.get("method") is None:
        return _add_null_subpixel_rays(sensor)
    method, kx, ky = _parse_sub_pixel_ray_args(sub_pixel_ray_args)
    px, wx = method(X.size, **kx)  # one set of samples per pixel and image axis
    py, wy = method(Y.size, **ky)
    pert_x = np.repeat(np.asarray(px)[..., np.newaxis] * x_resolution / 2.0, np.shape(py)[-1], axis=-1)
    pert_y = np.repeat(np.asarray(py)[..., np.newaxis, :] * y_resolution / 2.0, np.shape(px)[-1], axis=-2)
    wbx = np.repeat(np.asarray(wx)[..., np.newaxis], np.shape(wy)[-1], axis=-1)
    wby = np.repeat(np.asarray(wy)[..., np.newaxis, :], np.shape(wx)[-1], axis=-2)
    nsx, nsy = pert_x.shape[-2], pert_y.shape[-1]
    rep = lambda a: np.repeat(np.repeat(a.ravel()[:, np.newaxis, np.newaxis], nsx, axis=-2), nsy, axis=-1).ravel()
    sensor["ray_x"] = (X.ravel()[:, np.newaxis, np.newaxis] + pert_x).ravel()
    sensor["ray_y"] = (Y.ravel()[:, np.newaxis, np.newaxis] + pert_y).ravel()
    sensor["ray_z"] = rep(Z)
    sensor["ray_mu"] = rep(MU)
    sensor["ray_phi"] = rep(PHI)
    sensor["pixel_index"] = np.repeat(np.repeat(np.arange(len(sensor["cam_mu"])), np.shape(wx)[-1]), np.shape(wy)[-1])
    sensor["ray_weight"] = (wbx * wby).ravel()
    sensor["use_subpixel_rays"] = True
    _check_ray_layout(sensor)
    sensor["attrs"].update({f"sub_pixel_ray_args_{k}": (v.__name__ if k == "method" else v)
                            for k, v in sub_pixel_ray_args.items()})
    return sensor


def perspective_projection(wavelength, fov, x_resolution, y_resolution, position_vector, lookat_vector, up_vector,
                           stokes="I", sub_pixel_ray_args=None) -> dict:
    """A pinhole camera at position_vector looking at lookat_vector with the
    given field of view (degrees) and x_resolution x y_resolution pixels
    (at3d/sensor.py:367-553): every ray starts at the camera position; its
    direction comes from the normalised image-plane coordinates through the
    inverse camera matrix and the camera rotation."""
    sub_pixel_ray_args = dict(sub_pixel_ray_args or {"method": None})

    def norm(v):
        return v / np.linalg.norm(v, axis=0)

    if int(x_resolution) != x_resolution or int(y_resolution) != y_resolution:
        raise ValueError("x_resolution and y_resolution are integers >= 1")
    nx, ny = int(x_resolution), int(y_resolution)
    position = np.array(position_vector, dtype=np.float32)
    lookat = np.array(lookat_vector, dtype=np.float32)
    up = np.array(up_vector)
    zaxis = norm(lookat - position)
    xaxis = norm(np.cross(up, zaxis))
    yaxis = np.cross(zaxis, xaxis)
    rot = np.stack((xaxis, yaxis, zaxis), axis=1)
    M = max(nx, ny)
    R = np.array([nx, ny]) / M
    dy, dx = 2 * R[1] / ny, 2 * R[0] / nx
    xs, ys, zs = np.meshgrid(np.linspace(-R[0] + dx / 2, R[0] - dx / 2, nx),
                             np.linspace(-R[1] + dy / 2, R[1] - dy / 2, ny), 1.0)
    focal = 1.0 / np.tan(np.deg2rad(fov) / 2.0)
    k = np.array([[focal, 0, 0], [0, focal, 0], [0, 0, 1]], dtype=np.float32)
    inv_k = np.linalg.inv(k)

    def directions(hx, hy, hz):
        xc, yc, zc = norm(rot @ (inv_k @ np.stack([hx, hy, hz])))
        return -zc.astype(np.float64), (np.arctan2(yc, xc) + np.pi).astype(np.float64)

    mu, phi = directions(xs.ravel(), ys.ravel(), zs.ravel())
    npix = nx * ny
    sensor = make_sensor_dataset(np.full(npix, position[0], np.float32), np.full(npix, position[1], np.float32),
                                 np.full(npix, position[2], np.float32), mu, phi, stokes, wavelength,
                                 fill_ray_variables=False)
    sensor["image_shape"] = [nx, ny]
    sensor["attrs"] = {"projection": "Perspective", "fov_deg": fov,
                       "fov_x_deg": np.rad2deg(2 * np.arctan(R[0] / focal)),
                       "fov_y_deg": np.rad2deg(2 * np.arctan(R[1] / focal)), "x_resolution": x_resolution,
                       "y_resolution": y_resolution, "position": position, "lookat": lookat,
                       "rotation_matrix": rot.ravel(), "sensor_to_camera_transform_matrix": k.ravel()}
    if sub_pixel_ray_args.get("method") is None:
        return _add_null_subpixel_rays(sensor)
    method, kx, ky = _parse_sub_pixel_ray_args(sub_pixel_ray_args)
    px, wx = method(xs.size, **kx)
    py, wy = method(ys.size, **ky)
    pert_x = np.repeat(np.asarray(px)[..., np.newaxis] * dx / 2.0, np.shape(py)[-1], axis=-1)
    pert_y = np.repeat(np.asarray(py)[..., np.newaxis, :] * dy / 2.0, np.shape(px)[-1], axis=-2)
    wbx = np.repeat(np.asarray(wx)[..., np.newaxis], np.shape(wy)[-1], axis=-1)
    wby = np.repeat(np.asarray(wy)[..., np.newaxis, :], np.shape(wx)[-1], axis=-2)
    nsx, nsy = pert_x.shape[-2], pert_y.shape[-1]
    xr_ = (xs.ravel()[:, np.newaxis, np.newaxis] + pert_x).ravel()
    yr_ = (ys.ravel()[:, np.newaxis, np.newaxis] + pert_y).ravel()
    zr_ = np.repeat(np.repeat(zs.ravel()[:, np.newaxis, np.newaxis], nsx, axis=-2), nsy, axis=-1).ravel()
    rmu, rphi = directions(xr_, yr_, zr_)
    n = rmu.size
    sensor["ray_mu"], sensor["ray_phi"] = rmu, rphi
    sensor["ray_x"] = np.full(n, position[0], np.float32).astype(np.float64)
    sensor["ray_y"] = np.full(n, position[1], np.float32).astype(np.float64)
    sensor["ray_z"] = np.full(n, position[2], np.float32).astype(np.float64)
    sensor["pixel_index"] = np.repeat(np.repeat(np.arange(npix), np.shape(wx)[-1]), np.shape(wy)[-1])
    sensor["ray_weight"] = (wbx * wby).ravel()
    sensor["use_subpixel_rays"] = True
    _check_ray_layout(sensor)
    sensor["attrs"].update({f"sub_pixel_ray_args_{k}": (v.__name__ if k == "method" else v)
                            for k, v in sub_pixel_ray_args.items()})
    return sensor


def domaintop_projection(wavelength, bounding_box, x_resolution, y_resolution, azimuth, zenith, x_offset=0.0,
                         y_offset=0.0, stokes="I", sub_pixel_ray_args=None) -> dict:
    """A nadir orthographic grid of pixels on the domain top, shifted by the
    offsets, whose rays all take the given view direction (SHDOM's
    default radiance output; at3d/sensor.py:555-622)."""
    sensor = orthographic_projection(wavelength, bounding_box, x_resolution, y_resolution, 0.0, 0.0,
                                     altitude="TOA", stokes=stokes, sub_pixel_ray_args=sub_pixel_ray_args)
    for k in ("cam_x", "ray_x"):
        sensor[k] = sensor[k] + x_offset
    for k in ("cam_y", "ray_y"):
        sensor[k] = sensor[k] + y_offset
    for k in ("cam_mu", "ray_mu"):
        sensor[k] = np.full_like(sensor[k], np.cos(np.deg2rad(zenith)))
    for k in ("cam_phi", "ray_phi"):
        sensor[k] = np.full_like(sensor[k], np.deg2rad(azimuth))
    sensor["attrs"].update({"projection": "DomainTop", "projection_azimuth": azimuth, "projection_zenith": zenith})
    return sensor


def _check_ray_layout(sensor: dict):
    n = len(sensor["ray_mu"])
    for k in ("ray_x", "ray_y", "ray_z", "ray_phi", "pixel_index", "ray_weight"):
        if len(sensor[k]) != n:
            raise ValueError(f"sub-pixel ray variable '{k}' has {len(sensor[k])} entries, expected {n}")


def average_subpixel_rays(pixel_index, weighted_stokes, npixels):
    """AVERAGE_SUBPIXEL_RAYS (src/util.f90:484-519): observables[s, p] is the
    sum of weighted_stokes[s, r] over the rays r with pixel_index[r] == p.
    weighted_stokes is [nstokes, nrays] (ray weight already applied) or
    [nrays]; the result is FP64 with the same leading shape."""
    ws = np.asarray(weighted_stokes, np.float64)
    idx = np.asarray(pixel_index)
    if idx.min(initial=0) < 0 or idx.max(initial=-1) >= npixels:
        raise ValueError("pixel_index out of range")
    if ws.ndim == 1:
        out = np.zeros(npixels, np.float64)
        np.add.at(out, idx, ws)
        return out
    out = np.zeros((ws.shape[0], npixels), np.float64)
    for s in range(ws.shape[0]):
        np.add.at(out[s], idx, ws[s])
    return out


def calculate_observables(sensor: dict, rendered_rays: dict) -> dict:
    """Pixel values of the rendered rays (SensorsDict._calculate_observables,
    at3d/containers.py:600-650): each requested Stokes component of the
    rays ('I', 'Q', 'U' from integrate_to_sensor) times the ray weights,
    summed per pixel.  Writes the pixel arrays into the sensor and returns it."""
    names = [s for s, on in zip(STOKES_NAMES, sensor["stokes"]) if on and s in rendered_rays]
    npix = len(sensor["cam_mu"])
    w = np.asarray(sensor["ray_weight"], np.float64)
    if not sensor.get("use_subpixel_rays", False):
        for s in names:
            sensor[s] = w * np.asarray(rendered_rays[s], np.float64)
        return sensor
    ws = np.stack([w * np.asarray(rendered_rays[s], np.float64) for s in names])
    obs = average_subpixel_rays(sensor["pixel_index"], ws, npix)
    for i, s in enumerate(names):
        sensor[s] = obs[i]
    return sensor
