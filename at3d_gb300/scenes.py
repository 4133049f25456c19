"""Seeded synthetic scenes for the benchmark configurations.

There is no public dataset behind the hot path's benchmark: every field is
drawn from ``numpy.random.default_rng(seed)`` with the shapes and value
distributions of the workload descriptions:

* ``cloud_blob``: scalar solar scene on a 32x32x24 periodic grid
  (dx=dy=0.02 km, dz=0.04 km), NMU=8/NPHI=16; a 3D Gaussian cloud blob
  (peak 20/km, sigma 0.15 km) times lognormal noise (sigma 0.3), ssa
  0.999999, Henyey-Greenstein g=0.85 as 64 Legendre terms, plus a Rayleigh
  layer (0.01/km, ssa 1); Lambertian albedo 0.05, sun zenith 30 deg.
* ``cloud_field``: 128x128x64 grid (dz=0.025 km), NMU=16/NPHI=32, a k^-5/3
  Gaussian random field thresholded to 30% cloud fraction, in-cloud
  lognormal extinction (mean 30/km, log-sigma 0.5), per-wavelength ssa and
  HG g from the four-wavelength set, 128 Legendre terms.
* ``polarized_blob``: NSTOKES=3 scene on a 64x64x40 periodic grid with the
  geometry of ``cloud_blob`` (dx=dy=0.02 km, dz=0.04 km), NMU=8/NPHI=16; the
  blob extinction field of ``cloud_blob`` (seeded); one phase matrix of six
  64-term Wigner-function series, the 50/50 mix of a Rayleigh matrix and a
  Henyey-Greenstein-derived matrix (g=0.8, linear depolarisation 0.03);
  Lambertian albedo 0.1, sun zenith 45 deg.
* ``mie_cloud``: a water cloud from microphysics through Mie tables
  (gamma size distributions, veff 0.1, water index 1.331 - 1.6e-8 i at
  0.672 um): condensate density a Gaussian blob (sigma a quarter of the
  domain width, peak 0.1 g/m^3) times lognormal noise (sigma 0.3),
  effective radius rising linearly from 6 um at the base to 14 um at the
  top, on a 24x24x16 open grid
  (dx = dz = 0.04 km), plus a Rayleigh layer; NMU=8/NPHI=16, Lambertian
  albedo 0.05, sun zenith 30 deg; scalar (a1 rows) or NSTOKES=3 (all six).
* ``orthographic_views``: parallel rays on a regular pixel grid at the domain
  top for a list of view zenith angles in the azimuth-0 plane; mu and phi
  point towards the sensor (at3d/sensor.py:44-47 convention).
"""
from __future__ import annotations

import numpy as np

from ._abi import NumericalParams, Problem, Species
from .medium import henyey_greenstein_legcoef, hg_matrix_legcoef6, rayleigh_legcoef, rayleigh_legcoef6

VIEW_ZENITHS = (0.0, 26.1, -26.1, 45.6, -45.6, 60.0, -60.0, 70.5, -70.5)
FIELD_SSA = (0.99999, 0.9999, 0.999, 0.99)
FIELD_G = (0.85, 0.84, 0.82, 0.80)


def cloud_blob(seed: int = 1, nx: int = 32, ny: int = 32, nz: int = 24, dx: float = 0.02,
               dz: float = 0.04, boundary: str = "periodic", nmu: int = 8, nphi: int = 16,
               solacc: float = 1e-5) -> Problem:
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * dx
    y = np.arange(ny) * dx
    z = (np.arange(nz) * dz).astype(np.float32)
    cx, cy, cz = nx * dx / 2, ny * dx / 2, z[-1] / 2
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    r2 = (X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2
    ln = rng.lognormal(mean=0.0, sigma=0.3, size=(nx, ny, nz))
    ext = (20.0 * np.exp(-r2 / (2 * 0.15 ** 2)) * ln).astype(np.float32)
    cloud = Species(extinction=ext, ssalb=np.full_like(ext, 0.999999),
                    legcoef=henyey_greenstein_legcoef(0.85, 64))
    ray_ext = np.full_like(ext, 0.01)
    rayleigh = Species(extinction=ray_ext, ssalb=np.ones_like(ext), legcoef=rayleigh_legcoef(0.86))
    params = NumericalParams(num_mu_bins=nmu, num_phi_bins=nphi, solution_accuracy=solacc,
                             split_accuracy=0.0, x_boundary_condition=boundary,
                             y_boundary_condition=boundary)
    return Problem(delx=dx, dely=dx, zlevels=z, species=[cloud, rayleigh],
                   solarmu=-float(np.cos(np.deg2rad(30.0))), solaraz=0.0, solarflux=1.0,
                   surface_albedo=0.05, params=params)


def polarized_matrix(nterms: int = 64, g: float = 0.8, depol: float = 0.03) -> np.ndarray:
    """[6, nterms] phase matrix: 0.5 Rayleigh + 0.5 HG-derived (a1 a2 a3 a4 b1 b2)."""
    ray = np.zeros((6, nterms), np.float32)
    ray[:, :3] = rayleigh_legcoef6(depol)
    return (0.5 * ray + 0.5 * hg_matrix_legcoef6(g, depol, nterms)).astype(np.float32)


def polarized_blob(seed: int = 1, nx: int = 64, ny: int = 64, nz: int = 40, dx: float = 0.02,
                   dz: float = 0.04, boundary: str = "periodic", nmu: int = 8, nphi: int = 16,
                   solacc: float = 1e-5, ssa: float = 0.999999) -> Problem:
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * dx
    y = np.arange(ny) * dx
    z = (np.arange(nz) * dz).astype(np.float32)
    cx, cy, cz = nx * dx / 2, ny * dx / 2, z[-1] / 2
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    r2 = (X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2
    ln = rng.lognormal(mean=0.0, sigma=0.3, size=(nx, ny, nz))
    ext = (20.0 * np.exp(-r2 / (2 * 0.15 ** 2)) * ln).astype(np.float32)
    cloud = Species(extinction=ext, ssalb=np.full_like(ext, ssa), legcoef=polarized_matrix())
    params = NumericalParams(num_mu_bins=nmu, num_phi_bins=nphi, solution_accuracy=solacc,
                             split_accuracy=0.0, x_boundary_condition=boundary,
                             y_boundary_condition=boundary)
    return Problem(delx=dx, dely=dx, zlevels=z, species=[cloud],
                   solarmu=-float(np.cos(np.deg2rad(45.0))), solaraz=0.0, solarflux=1.0,
                   surface_albedo=0.1, params=params, num_stokes=3)


def powerlaw_field(rng, shape, fraction: float):
    """Boolean cloud mask from a k^-5/3 Gaussian random field thresholded at
    the (1-fraction) quantile, plus the field itself."""
    noise = rng.standard_normal(shape)
    k = [np.fft.fftfreq(n) for n in shape]
    K = np.sqrt(sum(np.meshgrid(*[kk ** 2 for kk in k], indexing="ij")))
    K[0, 0, 0] = np.inf
    amp = K ** (-5.0 / 6.0)  # power spectrum k^-5/3 -> amplitude k^-5/6
    f = np.real(np.fft.ifftn(np.fft.fftn(noise) * amp))
    thr = np.quantile(f, 1.0 - fraction)
    return f > thr, f


def cloud_field(seed: int = 2, wavelength_index: int = 0, nx: int = 128, ny: int = 128, nz: int = 64,
                dx: float = 0.02, dz: float = 0.025, fraction: float = 0.3, mean_ext: float = 30.0,
                boundary: str = "open", nmu: int = 16, nphi: int = 32, nleg: int = 128,
                solacc: float = 1e-4, ssa=None, g=None) -> Problem:
    rng = np.random.default_rng(seed)
    mask, _ = powerlaw_field(rng, (nx, ny, nz), fraction)
    sig = 0.5
    ln = rng.lognormal(mean=np.log(mean_ext) - 0.5 * sig ** 2, sigma=sig, size=(nx, ny, nz))
    ext = np.where(mask, ln, 0.0).astype(np.float32)
    ssa = FIELD_SSA[wavelength_index] if ssa is None else ssa
    g = FIELD_G[wavelength_index] if g is None else g
    cloud = Species(extinction=ext, ssalb=np.full_like(ext, ssa), legcoef=henyey_greenstein_legcoef(g, nleg))
    z = (np.arange(nz) * dz).astype(np.float32)
    params = NumericalParams(num_mu_bins=nmu, num_phi_bins=nphi, solution_accuracy=solacc,
                             split_accuracy=0.0, x_boundary_condition=boundary,
                             y_boundary_condition=boundary)
    return Problem(delx=dx, dely=dx, zlevels=z, species=[cloud],
                   solarmu=-float(np.cos(np.deg2rad(30.0))), solaraz=0.0, solarflux=1.0,
                   surface_albedo=0.05, params=params)


def mie_poly_table(wavelength: float = 0.672, reff=(4.0, 20.0, 17), veff=(0.09, 0.11),
                   max_radius: float = 30.0, refractive_index: complex = 1.331 - 1.6e-8j):
    """Poly table of water spheres, gamma distributions on a logarithmic
    effective-radius grid (min, max, points) and the given veff points."""
    from .mie import get_mono_table, get_poly_table
    from .size_distribution import gamma, get_size_distribution_grid
    mono = get_mono_table("Water", (wavelength, wavelength), minimum_effective_radius=reff[0],
                          max_integration_radius=max_radius, refractive_index=refractive_index, verbose=False)
    grid = get_size_distribution_grid(
        mono.radius, size_distribution_function=gamma, particle_density=1.0,
        reff={"coord_min": reff[0], "coord_max": reff[1], "npoints": reff[2], "spacing": "logarithmic"},
        veff=np.asarray(veff, np.float64))
    return get_poly_table(grid, mono)


def mie_microphysics(seed: int = 1, nx: int = 24, ny: int = 24, nz: int = 16, dx: float = 0.04,
                     dz: float = 0.04, peak: float = 0.1, reff=(6.0, 14.0), veff: float = 0.1) -> dict:
    """Density [g/m^3], reff and veff on the property grid."""
    rng = np.random.default_rng(seed)
    x, y, z = np.arange(nx) * dx, np.arange(ny) * dx, np.arange(nz) * dz
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    r2 = (X - nx * dx / 2) ** 2 + (Y - ny * dx / 2) ** 2 + (Z - z[-1] / 2) ** 2
    density = peak * np.exp(-r2 / (2 * (0.25 * nx * dx) ** 2)) * rng.lognormal(0.0, 0.3, (nx, ny, nz))
    re = reff[0] + (reff[1] - reff[0]) * Z / max(z[-1], 1e-6)
    return {"density": density, "reff": re, "veff": np.full_like(density, veff)}


def mie_cloud(seed: int = 1, nx: int = 24, ny: int = 24, nz: int = 16, dx: float = 0.04, dz: float = 0.04,
              boundary: str = "open", nmu: int = 8, nphi: int = 16, solacc: float = 1e-5,
              num_stokes: int = 1, poly_table=None, microphysics=None) -> Problem:
    """Water cloud whose optical properties come from Mie tables through
    ``table_to_grid``, plus a Rayleigh layer."""
    from .medium import table_to_grid
    poly = mie_poly_table() if poly_table is None else poly_table
    micro = mie_microphysics(seed, nx, ny, nz, dx, dz) if microphysics is None else microphysics
    if np.shape(micro["density"]) != (nx, ny, nz):
        raise ValueError(f"microphysics of shape {np.shape(micro['density'])} for a {nx}x{ny}x{nz} grid")
    cloud = table_to_grid(micro, poly, num_stokes=num_stokes)
    ray_ext = np.full((nx, ny, nz), 0.01, np.float32)
    ray_leg = rayleigh_legcoef6(0.03) if num_stokes == 3 else rayleigh_legcoef(0.672)
    rayleigh = Species(extinction=ray_ext, ssalb=np.ones_like(ray_ext), legcoef=ray_leg)
    params = NumericalParams(num_mu_bins=nmu, num_phi_bins=nphi, solution_accuracy=solacc,
                             split_accuracy=0.0, x_boundary_condition=boundary,
                             y_boundary_condition=boundary)
    return Problem(delx=dx, dely=dx, zlevels=(np.arange(nz) * dz).astype(np.float32), species=[cloud, rayleigh],
                   solarmu=-float(np.cos(np.deg2rad(30.0))), solaraz=0.0, solarflux=1.0,
                   surface_albedo=0.05, params=params, num_stokes=num_stokes)


def orthographic_views(problem: Problem, npix_x: int, npix_y: int, zeniths=VIEW_ZENITHS):
    """Ray arrays (x, y, z, mu, phi) for parallel views covering the domain."""
    npx, npy, npz = problem.shape
    lx, ly = npx * problem.delx, npy * problem.dely
    xs = (np.arange(npix_x) + 0.5) * lx / npix_x
    ys = (np.arange(npix_y) + 0.5) * ly / npix_y
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    ztop = float(problem.zlevels[-1])
    out = [[], [], [], [], []]
    for zen in zeniths:
        mu = np.cos(np.deg2rad(abs(zen)))
        phi = 0.0 if zen >= 0 else np.pi
        out[0].append(X.ravel()); out[1].append(Y.ravel())
        out[2].append(np.full(X.size, ztop)); out[3].append(np.full(X.size, mu))
        out[4].append(np.full(X.size, phi))
    return tuple(np.concatenate(a) for a in out)


SERVING_GRIDS = ((32, 32, 24), (64, 64, 32), (96, 96, 48), (128, 128, 64))
SERVING_VIEWS = (0.0, 26.1, -26.1, 45.6, -45.6)


def request_mix(seed: int, n: int, grids=SERVING_GRIDS, max_wavelengths: int = 8, solacc: float = 1e-4):
    """A seeded stream of serving requests: each one a power-law cloud field on
    a grid drawn uniformly from ``grids``, NMU/NPHI 8/16 or 16/32, 1 to
    ``max_wavelengths`` wavelengths (one problem each, sharing the field),
    cloud fraction 10-50%, mean in-cloud extinction 10-40/km, HG g 0.75-0.88,
    and a 32x32 to 64x64-pixel render at 5 view zeniths.  Returns a list of
    (problems, rays) pairs."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx, ny, nz = grids[rng.integers(len(grids))]
        nmu, nphi = (8, 16) if rng.integers(2) == 0 else (16, 32)
        nw = int(rng.integers(1, max_wavelengths + 1))
        frac = float(rng.uniform(0.1, 0.5))
        mext = float(rng.uniform(10.0, 40.0))
        g0 = float(rng.uniform(0.75, 0.88))
        fseed = int(rng.integers(1 << 30))
        base = cloud_field(seed=fseed, nx=nx, ny=ny, nz=nz, fraction=frac, mean_ext=mext, nmu=nmu, nphi=nphi,
                           nleg=64, solacc=solacc, ssa=FIELD_SSA[0], g=g0)
        ext = base.species[0].extinction
        pbs = []
        for w in range(nw):
            ssa = FIELD_SSA[w % len(FIELD_SSA)]
            g = max(0.70, g0 - 0.01 * w)
            sp = Species(extinction=ext, ssalb=np.full_like(ext, ssa), legcoef=henyey_greenstein_legcoef(g, 64))
            pbs.append(Problem(delx=base.delx, dely=base.dely, zlevels=base.zlevels, species=[sp],
                               solarmu=base.solarmu, solaraz=base.solaraz, solarflux=base.solarflux,
                               surface_albedo=base.surface_albedo, params=base.params))
        npix = int(rng.choice([32, 48, 64]))
        out.append((pbs, orthographic_views(pbs[0], npix, npix, zeniths=SERVING_VIEWS)))
    return out
