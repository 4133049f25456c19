"""Grid helpers on the host: resampling with the reference's NaN filling,
and the merging of z coordinates (at3d/grid.py:96-306)."""
import numpy as np
import pytest

from at3d_gb300.grid import (_fill_axis, combine_z_coordinates, from_scatterer, make_grid,
                             merge_two_z_coordinates, resample_onto_grid)


def test_fill_axis_backward_then_forward():
    a = np.array([[np.nan, 1.0, np.nan, np.nan, 4.0, np.nan]])
    assert np.array_equal(_fill_axis(a, 1), [[1.0, 1.0, 4.0, 4.0, 4.0, 4.0]])
    assert np.all(np.isnan(_fill_axis(np.full((2, 3), np.nan), 1)))


def test_resample_linear_fields_exactly():
    """A field linear in x, y, z is reproduced exactly inside the data's
    extent and held at the edge value outside it; density is zero outside."""
    xs, ys, zs = np.linspace(0, 1.0, 6), np.linspace(0, 0.8, 5), np.linspace(0.2, 1.2, 7)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    f = 1 + 2 * X - Y + 3 * Z
    grid = make_grid(0.05, 21, 0.05, 17, np.linspace(0.0, 1.4, 15))
    out = resample_onto_grid(grid, {"x": xs, "y": ys, "z": zs, "reff": f, "density": np.ones_like(f)})
    gX, gY, gZ = np.meshgrid(grid.x, grid.y, grid.z, indexing="ij")
    inside = (gZ >= 0.2) & (gZ <= 1.2 - 1e-6)     # the grid z is single precision
    assert np.allclose(out["reff"][inside], (1 + 2 * gX - gY + 3 * gZ)[inside])
    assert np.allclose(out["reff"][gZ < 0.2], (1 + 2 * gX - gY + 3 * 0.2)[gZ < 0.2])      # filled from above
    assert np.all(out["density"][~inside] == 0.0) and np.allclose(out["density"][inside], 1.0)
    assert out["delx"] == 0.05 and out["reff"].shape == (21, 17, 15)


def test_resample_fills_missing_values():
    xs, ys, zs = np.arange(4.0), np.arange(3.0), np.arange(5.0)
    reff = np.full((4, 3, 5), 10.0)
    reff[1:3, :, 2] = np.nan          # missing where there is no cloud
    dens = np.ones((4, 3, 5)); dens[1:3, :, 2] = np.nan
    out = resample_onto_grid(make_grid(1.0, 4, 1.0, 3, zs), {"x": xs, "y": ys, "z": zs, "reff": reff,
                                                               "density": dens})
    assert np.allclose(out["reff"], 10.0) and np.all(out["density"][1:3, :, 2] == 0.0)
    prof = resample_onto_grid(make_grid(1.0, 2, 1.0, 2, zs), {"x": xs, "y": ys, "z": zs, "temperature": 280 - zs})
    assert np.allclose(prof["temperature"][1, 1], 280 - zs)


def test_merge_z_coordinates():
    a = np.array([0.0, 0.5, 1.0, 1.5, 2.0])
    b = np.array([1.0, 1.1, 1.2, 1.3, 1.4, 1.5, 3.0])
    m = merge_two_z_coordinates(a, b)
    # below the overlap a's levels, above it b's, inside it the finer b's
    assert np.array_equal(m, [0.0, 0.5, 1.0, 1.1, 1.2, 1.3, 1.4, 1.5, 3.0])
    assert np.array_equal(combine_z_coordinates([a]), a)
    assert np.all(np.diff(combine_z_coordinates([a, b, np.array([2.5, 4.0])])) > 0)
    with pytest.raises(ValueError):
        merge_two_z_coordinates([1.0, 0.5], b)
    with pytest.raises(TypeError):
        combine_z_coordinates(a)


def test_from_scatterer():
    xs, ys, zs = np.arange(3) * 0.1, np.arange(4) * 0.2, np.array([0.0, 0.3, 0.7])
    f = np.random.default_rng(0).uniform(size=(3, 4, 3))
    out = from_scatterer({"x": xs, "y": ys, "z": zs, "density": f})
    assert np.allclose(out["density"], f) and out["delx"] == pytest.approx(0.1)
