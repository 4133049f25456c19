"""Optical-property producers on the host (no GPU): the Lorenz-Mie table,
size distributions, the poly table and table_to_grid.

The reference's Mie tables are netCDF files this environment cannot read, and
its Fortran has no compiler here, so the Mie routine is pinned on published
values and physical identities instead:

* Bohren and Huffman's worked example (m = 1.55, x = 5.213):
  Qext = Qsca = 3.10543 and Qback = 2.92534 (five digits as printed);
* the Rayleigh limit x -> 0: Qsca = 8/3 x^4 |K|^2, Qabs = 4 x Im(K) with
  K = (m^2 - 1)/(m^2 + 2), and the phase matrix of Rayleigh scattering
  without depolarisation (a1 = (1, 0, 1/2), a2_2 = 3, a4_1 = 3/2,
  b1_2 = sqrt(3/2));
* the extinction paradox Qext -> 2 for large spheres;
* a1_0 of every radius equal to the scattering cross section (the phase
  function integrates to one), energy conservation Qext = Qsca without
  absorption, a non-negative phase function.
"""
import os

import numpy as np
import pytest

from at3d_gb300 import mie, size_distribution as sd
from at3d_gb300.medium import rayleigh_legcoef6, table_to_grid


@pytest.fixture(scope="module")
def built():
    from at3d_gb300 import _lib
    from at3d_gb300.build import build
    if not os.path.exists(_lib.LIB):
        build()
    return True


def test_bohren_huffman_example(built):
    wl, r = 0.6328, 0.525
    ext, sca, nleg, leg = mie.mie_mono(wl, 1.55 + 0j, [r], 200)
    area = np.pi * r * r
    x = 2 * np.pi * r / wl
    assert abs(ext[0] / area - 3.10543) < 1e-5
    assert abs(sca[0] / area - 3.10543) < 1e-5
    l = np.arange(leg.shape[1])
    p1_back = np.pi / wl ** 2 * np.sum(leg[0, :, 0].astype(np.float64) * (-1.0) ** l)
    assert abs(4 * p1_back / x ** 2 - 2.92534) < 1e-4
    # nleg = 2 x series length, series length int(x + 6.5 x^0.3334 + 2)
    assert nleg[0] == 2 * int(x + 6.5 * x ** 0.3334 + 2)


def test_rayleigh_limit(built):
    wl, r, m = 0.5, 0.0005, 1.5 - 0.01j
    ext, sca, nleg, leg = mie.mie_mono(wl, m, [r], 16)
    x = 2 * np.pi * r / wl
    mb = np.conj(m)
    K = (mb * mb - 1) / (mb * mb + 2)
    area = np.pi * r * r
    assert abs(sca[0] / area / (8 / 3 * x ** 4 * abs(K) ** 2) - 1) < 1e-3
    assert abs((ext[0] - sca[0]) / area / (4 * x * K.imag) - 1) < 1e-3
    norm = leg[:, :3, 0] / sca[0]
    assert np.allclose(norm, rayleigh_legcoef6(0.0), atol=1e-4)


def test_large_sphere_extinction_paradox(built):
    ext, sca, nleg, leg = mie.mie_mono(0.5, 1.33 + 0j, [150.0, 160.0], 4000)
    assert np.all(np.abs(ext / (np.pi * np.array([150.0, 160.0]) ** 2) - 2.0) < 0.02)
    x = 2 * np.pi * 150.0 / 0.5
    assert nleg[0] == 2 * int(x + 6.5 * x ** 0.3334 + 2) < 4000
    assert nleg[1] == 4000     # clipped at maxleg


def test_normalisation_and_positivity(built):
    radii = np.geomspace(0.05, 20.0, 60).astype(np.float32)
    ext, sca, nleg, leg = mie.mie_mono(0.67, 1.33 - 0j, radii, 600)
    assert np.allclose(leg[0, 0] / sca, 1.0, rtol=2e-6)
    assert np.allclose(ext, sca, rtol=2e-5)                  # no absorption
    ext_a, sca_a, _, leg_a = mie.mie_mono(0.67, 1.33 - 0.01j, radii, 600)
    assert np.all(sca_a < ext_a)
    mu, w = np.polynomial.legendre.leggauss(1200)
    for k in (0, 30, 59):
        f = np.polynomial.legendre.legval(mu, leg[0, :, k].astype(np.float64) / sca[k])
        assert f.min() > -1e-3 * f.max()
        assert abs(0.5 * np.dot(w, f) - 1.0) < 1e-5
        g = leg[0, 1, k] / (3 * leg[0, 0, k])
        assert -1.0 < g < 1.0
        # |b1| <= a1 at every angle: the degree of polarisation stays below one
        d20 = np.zeros_like(mu)
        # b1 expansion in d^l_20: evaluate by recurrence
        dm1, d = np.zeros_like(mu), np.sqrt(6) / 4 * (1 - mu * mu)
        for l in range(2, nleg[k] + 1):
            d20 += leg[4, l, k] * d
            q = (l + 1) ** 2 - 4
            d, dm1 = ((2 * l + 1) * mu * d - np.sqrt(l * l - 4) * dm1) / np.sqrt(q), d
        assert np.all(np.abs(d20) <= f * sca[k] * (1 + 1e-3) + 1e-3 * f.max() * sca[k])


def test_threads_do_not_change_results(built):
    radii = np.linspace(0.2, 8.0, 40).astype(np.float32)
    a = mie.mie_mono(0.86, 1.45 - 0.002j, radii, 200, n_threads=1)
    b = mie.mie_mono(0.86, 1.45 - 0.002j, radii, 200, n_threads=7)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def test_bad_arguments(built):
    with pytest.raises(ValueError, match="refractive index"):
        mie.mie_mono(0.5, 1.33 + 0.1j, [1.0], 10)
    with pytest.raises(ValueError, match="radii"):
        mie.mie_mono(0.5, 1.33, [0.0], 10)
    with pytest.raises(ValueError, match="Water"):
        mie.get_mono_table("Water", (0.5, 0.5), verbose=False)
    with pytest.raises(AttributeError):
        mie.get_mono_table("Ice", (0.5, 0.5), refractive_index=1.3, verbose=False)
    with pytest.raises(AttributeError, match="negative imaginary"):
        mie.get_mono_table("Aerosol", (0.5, 0.5), refractive_index=1.3 + 0.01j, verbose=False)


def test_radius_grid_and_band_centre():
    r = mie.get_sizes(4.0, 30.0, 0.672)
    assert r[0] == np.float32(0.08) and r[-2] < 30.0 <= r[-1]
    steps = np.diff(r.astype(np.float64))
    assert np.all(steps > 0) and steps.max() <= 0.002 * 30.0 * (1 + 1e-6)
    x = 2 * np.pi * r[:-1] / 0.672
    want = np.minimum(np.maximum(0.01, 0.03 * np.sqrt(x)) * 0.672 / (2 * np.pi), 0.06)
    assert np.allclose(steps, want, rtol=1e-4)
    assert mie.get_center_wavelen(0.672, 0.672) == pytest.approx(0.672)
    c = mie.get_center_wavelen(0.6, 0.8)
    assert 0.6 < c < 0.7 and abs(c * 1000 - round(c * 1000)) < 1e-3   # solar weights favour the short end
    assert mie.get_center_wavelen(3.5, 4.5) == pytest.approx(4.0, abs=1e-3)   # flat weights
    assert mie.maximum_legendre(30.0, 0.672) == int(np.round(2 * (280.5 + 4 * 280.5 ** 0.3334 + 2)))


@pytest.mark.parametrize("fn", [sd.gamma, sd.lognormal])
def test_size_distribution_normalisation(fn):
    radii = mie.get_sizes(4.0, 65.0, 0.672).astype(np.float64)
    reff = np.array([5.0, 10.0, 20.0])
    veff = np.array([0.05, 0.1, 0.2])
    nd = fn(radii, reff, veff).astype(np.float64)
    lwc = (1e-6 * nd * 4 * np.pi / 3 * radii[:, None] ** 3).sum(0)
    assert np.allclose(lwc, 1.0, rtol=1e-5)
    re = (nd * radii[:, None] ** 3).sum(0) / (nd * radii[:, None] ** 2).sum(0)
    assert np.all(np.abs(re / reff - 1) <= 1.0e-3 * (1 + 1e-4))
    # alpha and veff forms agree
    alpha = 1.0 / veff - 3.0 if fn is sd.gamma else np.sqrt(np.log(veff + 1.0))
    assert np.allclose(fn(radii, reff, alpha=alpha), nd, rtol=1e-6)
    ng = fn(radii, reff, veff, normalization="geometric_extinction").astype(np.float64)
    assert np.allclose(1e-3 * (2 * ng * np.pi * radii[:, None] ** 2).sum(0), 1.0, rtol=1e-5)
    nc = fn(radii, reff, veff, normalization="number_concentration").astype(np.float64)
    assert np.allclose(nc.sum(0), 1.0, rtol=1e-5)


def test_size_distribution_errors():
    r = np.linspace(0.1, 30, 300)
    with pytest.raises(ValueError, match="same length"):
        sd.gamma(r, [5.0, 6.0], veff=[0.1])
    with pytest.raises(ValueError, match="must be specified"):
        sd.lognormal(r, [5.0])
    with pytest.raises(ValueError, match="normalization"):
        sd.gamma(r, [5.0], veff=[0.1], normalization="mass")
    with pytest.raises(ValueError, match="cannot be achieved"):
        sd.gamma(r, [60.0], veff=[0.1])          # beyond the radius range


def test_size_distribution_grid_shapes():
    r = np.linspace(0.5, 40, 400)
    g = sd.get_size_distribution_grid(
        r, sd.gamma, reff={"coord_min": 5.0, "coord_max": 20.0, "npoints": 4, "spacing": "logarithmic",
                           "units": "micron"},
        veff=np.array([0.05, 0.1, 0.15]))
    assert g.number_density.shape == (400, 4, 3)
    assert list(g.coords) == ["reff", "veff"] and g.dims == ["radius", "reff", "veff"]
    assert np.allclose(g.coords["reff"], np.geomspace(5, 20, 4))
    assert g.attrs["distribution_type"] == "gamma" and g.attrs["reff_npoints"] == 4
    col = sd.gamma(r, [g.coords["reff"][2]], [0.15])[:, 0]
    assert np.allclose(g.number_density[:, 2, 2], col)


@pytest.fixture(scope="module")
def poly(built):
    mono = mie.get_mono_table("Water", (0.672, 0.672), minimum_effective_radius=4.0, max_integration_radius=30.0,
                              refractive_index=1.331 - 1.6e-8j, verbose=False)
    grid = sd.get_size_distribution_grid(
        mono.radius, sd.gamma, reff={"coord_min": 4.0, "coord_max": 20.0, "npoints": 9, "spacing": "logarithmic"},
        veff=np.array([0.09, 0.11]))
    return mono, grid, mie.get_poly_table(grid, mono)


def test_poly_table(poly):
    mono, grid, p = poly
    assert p.extinction.shape == (9, 2) and p.legcoef.shape == (6, mono.legendre.shape[1], 9, 2)
    assert np.allclose(p.legcoef[0, 0], 1.0, atol=1e-6)
    assert np.all((p.ssalb > 0.99999) & (p.ssalb <= 1.0))
    g = p.legcoef[0, 1] / 3
    assert np.all((g > 0.8) & (g < 0.9))                    # cloud droplets in the visible
    # extinction per g/m^3 = 750 <Qext> / reff [1/km], reff in um; Qext of cloud droplets ~ 2.0-2.2 here
    q = p.extinction * grid.coords["reff"][:, None] / 750.0
    assert np.all((q > 1.95) & (q < 2.3))
    # direct sums of the mono table
    nd = grid.number_density[:, 4, 1].astype(np.float64)
    assert p.extinction[4, 1] == pytest.approx(1e-3 * nd @ mono.extinction, rel=1e-6)
    assert p.ssalb[4, 1] == pytest.approx((nd @ mono.scatter) / (nd @ mono.extinction), rel=1e-6)
    leg = np.einsum("klr,r->kl", mono.legendre.astype(np.float64), nd) / (nd @ mono.scatter)
    assert np.allclose(p.legcoef[:, :, 4, 1], leg, atol=1e-6)
    last = np.flatnonzero(leg[0] > 0.5e-5).max()
    assert p.nleg[4, 1] == last
    assert np.array_equal(p.table_index, np.arange(18).reshape(9, 2))


def test_poly_table_interpolates_other_radii(poly):
    mono, grid, p = poly
    r = np.linspace(mono.radius.min(), mono.radius.max(), 3000)
    g2 = sd.get_size_distribution_grid(r, sd.gamma, reff=np.array([8.0, 12.0]), veff=np.array([0.1]))
    p2 = mie.get_poly_table(g2, mono)
    assert np.allclose(p2.legcoef[0, 0], 1.0, atol=1e-6)
    with pytest.raises(ValueError, match="outside of range"):
        g3 = sd.get_size_distribution_grid(np.linspace(1.0, 25.0, 100), sd.gamma, reff=np.array([8.0]),
                                           veff=np.array([0.1]))
        mie.get_poly_table(g3, mono)


def test_table_to_grid(poly):
    _, _, p = poly
    reff_ax = p.coords["reff"]
    shape = (3, 4, 5)
    rng = np.random.default_rng(0)
    micro = {"density": rng.uniform(0.0, 0.5, shape),
             "reff": rng.uniform(reff_ax[0] + 0.01, reff_ax[-1] - 0.01, shape),
             "veff": np.full(shape, 0.1)}
    sp = table_to_grid(micro, p)
    # linear interpolation along reff, midway in veff
    i = np.searchsorted(reff_ax, micro["reff"]) - 1
    t = (micro["reff"] - reff_ax[i]) / (reff_ax[i + 1] - reff_ax[i])
    e = 0.5 * (p.extinction[:, 0] + p.extinction[:, 1])
    w = 0.5 * (p.ssalb[:, 0] + p.ssalb[:, 1])
    assert np.allclose(sp.extinction, micro["density"] * ((1 - t) * e[i] + t * e[i + 1]), rtol=1e-5)
    assert np.allclose(sp.ssalb, (1 - t) * w[i] + t * w[i + 1], rtol=1e-6)
    # nearest table entry per coordinate, gathered into a compact 1-based table
    near_r = np.abs(reff_ax[None, :] - micro["reff"].reshape(-1, 1)).argmin(1)
    near_v = int(np.abs(p.coords["veff"] - 0.1).argmin())
    rows = sp.legcoef[sp.table_index[0].reshape(-1) - 1]
    assert np.array_equal(rows, p.legcoef[0, :, near_r, near_v])
    assert sp.table_index.shape == (1,) + shape and sp.phase_weights.shape == (1,) + shape
    assert sp.legcoef.shape[0] == len(np.unique(near_r))
    inv = table_to_grid(micro, p, inverse_mode=True)
    assert np.allclose(inv.extinction, (1 - t) * e[i] + t * e[i + 1], rtol=1e-5)
    pol = table_to_grid(micro, p, num_stokes=3)
    assert pol.legcoef.shape == (sp.legcoef.shape[0], 6, p.legcoef.shape[1])
    assert np.array_equal(pol.legcoef[:, 0], sp.legcoef)


def test_table_to_grid_errors(poly):
    _, _, p = poly
    shape = (2, 2, 2)
    micro = {"density": np.ones(shape), "reff": np.full(shape, 10.0), "veff": np.full(shape, 0.1)}
    with pytest.raises(KeyError):
        table_to_grid({"density": np.ones(shape), "reff": np.full(shape, 10.0)}, p)
    with pytest.raises(ValueError, match="within the range"):
        table_to_grid(dict(micro, reff=np.full(shape, 25.0)), p)
    with pytest.raises(ValueError, match="within the range"):
        table_to_grid(dict(micro, veff=np.full(shape, 0.09)), p)   # on the edge is outside
    with pytest.raises(ValueError, match="non-negative"):
        table_to_grid(dict(micro, density=-np.ones(shape)), p)


def test_mono_table_save_and_lookup(poly, tmp_path):
    mono, _, _ = poly
    mono.save(str(tmp_path / "water_mie_table_672.npz"))
    t = mie.get_mono_table("Water", (0.672, 0.672), minimum_effective_radius=4.0, max_integration_radius=30.0,
                           refractive_index=1.331 - 1.6e-8j, relative_dir=str(tmp_path), verbose=False)
    assert np.array_equal(t.legendre, mono.legendre) and t.attrs == mono.attrs
    # a different request is computed, not loaded
    t2 = mie.get_mono_table("Water", (0.672, 0.672), minimum_effective_radius=4.0, max_integration_radius=20.0,
                            refractive_index=1.331 - 1.6e-8j, relative_dir=str(tmp_path), verbose=False)
    assert t2.radius[-1] < t.radius[-1]


def test_band_average(built):
    t = mie.get_mono_table("Aerosol", (0.86, 0.87), minimum_effective_radius=1.0, max_integration_radius=2.0,
                           wavelength_averaging=True, wavelength_resolution=0.005, refractive_index=1.45 - 0.001j,
                           verbose=False)
    ws = [0.86, 0.865, 0.87]
    weights = [(1.19e8 / w ** 5) / (np.exp(1.439e4 / (w * 5800.0)) - 1) for w in np.float32(ws)]
    parts = [mie.mie_mono(float(np.float32(w)), 1.45 - 0.001j, t.radius, t.attrs["maximum_legendre"])
             for w in np.float32(ws)]
    ext = sum(wt * p[0].astype(np.float64) for wt, p in zip(weights, parts)) / sum(weights)
    assert np.allclose(t.extinction, ext, rtol=1e-5)
    assert np.allclose(t.legendre[0, 0], t.scatter, rtol=1e-5)


@pytest.fixture(scope="module")
def generator_tables(built):
    kw = dict(minimum_effective_radius=4.0, max_integration_radius=30.0, verbose=False)
    return {0.672: mie.get_mono_table("Water", (0.672, 0.672), refractive_index=1.331 - 1.6e-8j, **kw),
            0.86: mie.get_mono_table("Water", (0.86, 0.86), refractive_index=1.329 - 3e-7j, **kw)}


def _generator(tables, mode, **kw):
    from at3d_gb300.medium import OpticalPropertyGenerator
    return OpticalPropertyGenerator("cloud", tables, sd.gamma, interpolation_mode=mode,
                                    reff={"coord_min": 4.0, "coord_max": 20.0, "npoints": 17,
                                          "spacing": "logarithmic"},
                                    veff=np.array([0.09, 0.1, 0.11]), **kw)


def _micro(seed=0, shape=(5, 4, 3)):
    rng = np.random.default_rng(seed)
    return {"density": rng.uniform(0.0, 0.4, shape), "reff": rng.uniform(5.0, 18.0, shape),
            "veff": np.full(shape, 0.1)}


def test_generator_nearest_is_table_to_grid(generator_tables):
    g = _generator(generator_tables, "nearest")
    micro = _micro()
    out = g(micro)
    assert list(out) == [0.672, 0.86]
    for key in out:
        poly = mie.get_poly_table(g.size_distribution_grids[key], generator_tables[key])
        ref = table_to_grid(micro, poly)
        for f in ("extinction", "ssalb", "legcoef", "table_index", "phase_weights"):
            assert np.array_equal(getattr(out[key], f), getattr(ref, f)), f
    assert g(micro)[0.672] is out[0.672]        # the same microphysics returns the kept result


def test_generator_exact_few_tuples(generator_tables):
    """Fewer distinct (reff, veff) tuples than maxnphase: each point gets the
    poly properties of its own exact distribution."""
    g = _generator(generator_tables, "exact")
    micro = _micro()
    micro["reff"] = np.round(micro["reff"])           # a handful of distinct radii
    sp = g(micro)[0.672]
    r = np.unique(micro["reff"])
    assert sp.legcoef.shape[0] == r.size and sp.table_index.shape[0] == 1
    table = generator_tables[0.672]
    for k, re in enumerate(r):
        nd = sd.gamma(table.radius, [re], veff=[0.1])
        one = mie.get_poly_table(sd.SizeDistributionGrid(radius=table.radius, number_density=nd, coords={}), table)
        at = micro["reff"] == re
        assert np.all(sp.table_index[0][at] == k + 1)
        assert np.allclose(sp.extinction[at], micro["density"][at] * one.extinction[0], rtol=1e-6)
        assert np.allclose(sp.legcoef[k], one.legcoef[0, :, 0], rtol=1e-6, atol=1e-9)


def test_generator_exact_table_fallback(generator_tables):
    """More distinct radii than maxnphase: reff becomes a table, every point
    mixes the distributions at its bracketing grid radii with linear weights,
    so the extinction equals the linear interpolation of the poly table."""
    g = _generator(generator_tables, "exact", maxnphase=20)
    micro = _micro(1)
    sp = g(micro)[0.86]
    assert sp.table_index.shape[0] == 2 and sp.phase_weights.shape[0] == 2
    assert np.allclose(sp.phase_weights.sum(axis=0), 1.0)
    assert sp.legcoef.shape[0] <= 17
    near = _generator(generator_tables, "nearest")(micro)[0.86]
    assert np.allclose(sp.extinction, near.extinction, rtol=2e-5)
    assert np.allclose(sp.ssalb, near.ssalb, rtol=1e-6)
    reff_grid = g.size_distribution_grids[0.86].coords["reff"]
    lo = reff_grid[np.clip(np.digitize(micro["reff"], reff_grid), 1, reff_grid.size - 1) - 1]
    assert np.allclose(sp.phase_weights[0], (reff_grid[np.searchsorted(reff_grid, lo) + 1] - micro["reff"]) /
                       (reff_grid[np.searchsorted(reff_grid, lo) + 1] - lo), rtol=1e-5)


def test_generator_errors(generator_tables):
    from at3d_gb300.medium import OpticalPropertyGenerator
    with pytest.raises(ValueError, match="interpolation_mode"):
        _generator(generator_tables, "linear")
    with pytest.raises(TypeError):
        OpticalPropertyGenerator("c", [1], sd.gamma, reff=np.array([5.0, 6.0]))
    g = _generator(generator_tables, "exact", maxnphase=20)
    micro = _micro(2)
    with pytest.raises(KeyError):
        g({"density": micro["density"], "reff": micro["reff"]})
    with pytest.raises(ValueError, match="within the range"):
        g(dict(micro, reff=np.full(micro["reff"].shape, 25.0)))
    micro["veff"] = np.where(micro["reff"] > 10, 0.095, 0.105)   # two veff values, reff tabulated
    with pytest.raises(ValueError, match="not tabulated|maxnphase"):
        _generator(generator_tables, "exact", maxnphase=1)(micro)
