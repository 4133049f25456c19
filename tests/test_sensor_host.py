"""Sensor geometry (at3d/sensor.py mirrors) and pixel averaging of rendered
rays (average_subpixel_rays, src/util.f90:484-519), on the CPU."""
import numpy as np
import pytest

from at3d_gb300 import sensor as S
from at3d_gb300.grid import make_grid


def test_average_subpixel_rays_weights_and_pixels():
    rng = np.random.default_rng(0)
    npix, per = 7, 5
    idx = np.repeat(np.arange(npix), per)
    w = rng.uniform(0.1, 1.0, idx.size)
    rad = rng.uniform(0.0, 2.0, (3, idx.size))
    out = S.average_subpixel_rays(idx, w * rad, npix)
    ref = np.array([[np.sum(w[idx == p] * rad[s, idx == p]) for p in range(npix)] for s in range(3)])
    assert out.shape == (3, npix) and np.allclose(out, ref, rtol=1e-14)
    # rays of one pixel need not be contiguous; unused pixels stay zero
    perm = rng.permutation(idx.size)
    assert np.allclose(S.average_subpixel_rays(idx[perm], (w * rad[0])[perm], npix + 2)[:npix], ref[0])
    assert S.average_subpixel_rays(idx, w * rad[0], npix + 2)[-1] == 0.0
    with pytest.raises(ValueError):
        S.average_subpixel_rays(idx, rad[0], npix - 1)


@pytest.mark.parametrize("method,kw", [(S.gaussian, {"degree": (2, 3)}), (S.uniform, {"nrays": 4}),
                                       (S.stochastic, {"nrays": (3, 2), "seed": 5})])
def test_orthographic_subpixel_rays(method, kw):
    grid = make_grid(0.05, 10, 0.05, 8, np.linspace(0, 1.0, 11))
    sen = S.orthographic_projection(0.67, grid, 0.1, 0.1, 0.0, 45.6, sub_pixel_ray_args=dict(method=method, **kw))
    npix = len(sen["cam_mu"])
    assert sen["use_subpixel_rays"] and npix == sen["image_shape"][0] * sen["image_shape"][1]
    nr = len(sen["ray_mu"])
    assert all(len(sen[k]) == nr for k in ("ray_x", "ray_y", "ray_z", "ray_phi", "pixel_index", "ray_weight"))
    # weights of each pixel sum to one; rays stay within half a pixel of their pixel
    wsum = S.average_subpixel_rays(sen["pixel_index"], sen["ray_weight"], npix)
    assert np.allclose(wsum, 1.0)
    dx = sen["ray_x"] - sen["cam_x"][sen["pixel_index"]]
    dy = sen["ray_y"] - sen["cam_y"][sen["pixel_index"]]
    assert np.all(np.abs(dx) <= 0.05 + 1e-12) and np.all(np.abs(dy) <= 0.05 + 1e-12)
    assert np.allclose(sen["ray_mu"], np.cos(np.deg2rad(45.6)))
    # a uniform field is reproduced exactly by the pixel average
    obs = S.calculate_observables(sen, {"I": np.full(nr, 3.0)})
    assert np.allclose(obs["I"], 3.0)


def test_orthographic_footprint():
    """The pixels cover the bounding box projected along the view onto the
    altitude plane, with one padding sample at the far edge."""
    grid = make_grid(0.02, 16, 0.02, 12, np.linspace(0, 0.5, 6))
    sen = S.orthographic_projection(0.86, grid, 0.04, 0.04, 0.0, 0.0)
    xs, ys = np.unique(sen["cam_x"]), np.unique(sen["cam_y"])
    assert np.isclose(xs[0], 0.0) and np.isclose(xs[-1], 0.32) and len(xs) == 9
    assert np.isclose(ys[-1], 0.24) and len(ys) == 7
    assert np.all(sen["cam_z"] == 0.5) and not sen["use_subpixel_rays"]
    # oblique view, photons travelling towards +x (azimuth 0): the bottom of the box projects
    # z tan(zenith) further along +x on the top plane, so the footprint grows on that side
    ob = S.orthographic_projection(0.86, grid, 0.04, 0.04, 0.0, 60.0)
    x_end = 0.30 + 0.5 * np.tan(np.deg2rad(60.0))
    assert np.isclose(np.min(ob["cam_x"]), 0.0)
    assert x_end - 1e-9 <= np.max(ob["cam_x"]) < x_end + 0.04 + 1e-9
    assert np.allclose(ob["cam_phi"], 0.0) and np.allclose(ob["cam_mu"], 0.5)


def test_perspective_geometry():
    sen = S.perspective_projection(0.86, 30.0, 8, 6, [0.5, 0.5, 5.0], [0.5, 0.5, 0.0], [0.0, 1.0, 0.0],
                                   sub_pixel_ray_args={"method": S.gaussian, "degree": 2})
    assert sen["image_shape"] == [8, 6] and len(sen["cam_mu"]) == 48 and len(sen["ray_mu"]) == 48 * 4
    # looking straight down: every ray points up towards the camera from below (mu > 0 towards the sensor),
    # all start at the camera, and the central rays are close to nadir
    assert np.all(sen["ray_mu"] > np.cos(np.deg2rad(21.0))) and np.all(sen["cam_mu"] < 1.0)
    assert np.all(sen["ray_z"] == 5.0) and np.allclose(sen["ray_x"], 0.5)
    assert np.allclose(S.average_subpixel_rays(sen["pixel_index"], sen["ray_weight"], 48), 1.0)
    # the field of view bounds the widest ray: half the diagonal of the normalised image plane
    half = np.rad2deg(np.arctan(np.hypot(1.0, 0.75) * np.tan(np.deg2rad(15.0))))
    assert np.max(np.rad2deg(np.arccos(sen["cam_mu"]))) <= half + 1e-6


def test_domaintop_and_make_sensor_dataset():
    grid = make_grid(0.1, 5, 0.1, 5, [0.0, 0.5, 1.0])
    sen = S.domaintop_projection(0.86, grid, 0.1, 0.1, 90.0, 30.0, x_offset=0.05)
    assert np.allclose(sen["ray_mu"], np.cos(np.deg2rad(30.0))) and np.allclose(sen["ray_phi"], np.pi / 2)
    assert np.isclose(sen["cam_x"].min(), 0.05)
    with pytest.raises(ValueError):
        S.make_sensor_dataset([0.0], [0.0], [-1.0], [1.0], [0.0])
    with pytest.raises(ValueError):
        S.make_sensor_dataset([0.0], [0.0], [1.0], [0.0], [0.0])
    with pytest.raises(ValueError):
        S.make_sensor_dataset([0.0], [0.0], [1.0], [1.0], [0.0], stokes=["X"])
