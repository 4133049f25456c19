"""The scene of the reference's Verify_Lambertian_Surfaces test
(tests/test_shdom.py:29-68, :597-632): a 50x1x11 Rayleigh atmosphere at
0.85 um in independent-pixel mode over a variable Lambertian surface, NMU=16,
NPHI=32, solar mu0=-0.707, viewed by 19 upward directions at z=30 km; and
the same atmosphere over the RPV (Verify_RPV_Surfaces, :676-713) and, with
I, Q, U, the wave-Fresnel (Verify_WaveFresnel_Surfaces, :716-756) and Diner
(Verify_Diner_Surfaces, :759-800) surfaces."""
import numpy as np

from at3d_gb300._abi import NumericalParams, Problem, Species
from at3d_gb300.medium import rayleigh_extinction_profile, rayleigh_legcoef, rayleigh_legcoef6


def brdf_l1_problem():
    z = np.array([0, 3.0, 6.0, 9.0, 12.0, 15.0, 18.0, 21.0, 24.0, 27.0, 30.0], np.float32)
    temp = np.array([288.0, 269.0, 249.0, 230.0, 217.0, 217.0, 217.0, 218.0, 221.0, 224.0, 227.0])
    ext = rayleigh_extinction_profile(0.85, z, temp, surface_pressure=1013.25)
    ext = np.round(ext, 4).astype(np.float32)
    npx, npy = 50, 1
    ext3 = np.broadcast_to(ext[None, None, :], (npx, npy, len(z))).astype(np.float32)
    ray = Species(extinction=ext3, ssalb=np.ones_like(ext3), legcoef=rayleigh_legcoef(0.85))
    params = NumericalParams(num_mu_bins=16, num_phi_bins=32, solution_accuracy=1e-5,
                             spherical_harmonics_accuracy=0.0, split_accuracy=0.0,
                             x_boundary_condition="periodic", y_boundary_condition="periodic", ip_flag=3)
    albedo = np.linspace(0.0, 0.3 - (0.3 - 0.0) / 50.0, 50)[:, np.newaxis]
    return Problem(delx=0.02, dely=0.02, zlevels=z, species=[ray], solarmu=-0.707, solaraz=0.0,
                   solarflux=1.0, surface_albedo=albedo, surface_delx=0.02, surface_dely=0.04, params=params)


def brdf_l1_rays():
    x = np.linspace(0, 1.0 - 1.0 / 50, 50)
    mu = np.array([0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9] + [1.0] + [0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9][::-1])
    phi = np.array([180.0] * 9 + [0.0] * 10)
    return (np.tile(x, 19), np.zeros(950), np.full(950, 30.0), np.repeat(mu, 50), np.deg2rad(np.repeat(phi, 50)))


def _rayleigh6(wavelength=0.85):
    """The six-element Rayleigh matrix with the King depolarisation factor
    of RAYLEIGH_PHASE_FUNCTION (src/polarized/shdomsub4.f:2350-2386)."""
    a_k, b_k, c_k = 1.0469541, 3.2503153e-04, 3.8622851e-05
    w = np.float32(wavelength)
    fking = np.float32(a_k + b_k / np.float64(w) ** 2 + c_k / np.float64(w) ** 4)
    depol = float(np.float32(6.0 * (np.float64(fking) - 1.0) / (3.0 + 7.0 * np.float64(fking))))
    c = rayleigh_legcoef6(depol)
    c[0] = rayleigh_legcoef(wavelength)  # the same float32 arithmetic as the scalar row
    return c


def brdf_rpv_problem():
    pb = brdf_l1_problem()
    k = np.linspace(0.5, 1.0 - 0.5 / 50, 50)[:, np.newaxis]
    par = np.stack([np.full((50, 1), 0.1), k, np.full((50, 1), -0.24)], axis=-1).astype(np.float32)
    pb.surface_brdf, pb.surface_params = "R", par
    pb.surface_delx = pb.surface_dely = 0.02
    return pb


def brdf_ocean_problem():
    """Verify_Ocean_Unpolarized_Surfaces (tests/test_shdom.py:634-674 of the
    reference): the 6S ocean BRDF with the wind speed growing in x from 4
    to 11.84 m/s and no pigment, at 0.85 um."""
    pb = brdf_l1_problem()
    wind = np.linspace(4.0, 12.0 - 8.0 / 50, 50)[:, np.newaxis]
    par = np.stack([wind, np.zeros((50, 1))], axis=-1).astype(np.float32)
    pb.surface_brdf, pb.surface_params = "O", par
    pb.surface_delx, pb.surface_dely = 0.02, 0.04
    pb.wavelength = 0.85
    return pb


def brdf_wave_fresnel_problem():
    pb = brdf_l1_problem()
    wind = np.linspace(4.0, 12.0 - 8.0 / 50, 50)[:, np.newaxis]
    par = np.stack([np.full((50, 1), 1.33), np.zeros((50, 1)), wind], axis=-1).astype(np.float32)
    pb.surface_brdf, pb.surface_params = "W", par
    pb.surface_delx = pb.surface_dely = 0.02
    pb.num_stokes = 3
    pb.species[0].legcoef = _rayleigh6(0.85)
    return pb


def brdf_diner_problem():
    pb = brdf_l1_problem()
    zeta = np.linspace(0.0, 1.0 - 1.0 / 50, 50)[:, np.newaxis]
    one = np.ones((50, 1))
    par = np.stack([0.2 * one, 0.8 * one, 0.3 * one, zeta, -1.0 * one], axis=-1).astype(np.float32)
    pb.surface_brdf, pb.surface_params = "D", par
    pb.surface_delx = pb.surface_dely = 0.02
    pb.num_stokes = 3
    pb.species[0].legcoef = _rayleigh6(0.85)
    return pb


def gas_absorption_problem():
    """Verify_NonuniformGasAbsorption (tests/test_shdom.py:855-908 of the
    reference): the same grid with the Rayleigh extinction set to zero and a
    gaseous absorption growing linearly in x from 0 to 1 /km, overhead sun,
    Lambertian albedo 0.04, TRANSCUT 0; the nadir radiance at 30 km is
    exp(-tau) 0.04/pi exp(-tau) with tau = 30 km x absorption."""
    from at3d_gb300.medium import gas_species
    pb = brdf_l1_problem()
    ray = pb.species[0]
    ray.extinction = np.zeros_like(ray.extinction)
    gas = np.broadcast_to(np.linspace(0.0, 1.0, 50)[:, None, None], ray.extinction.shape).astype(np.float32)
    pb.species = [ray, gas_species(gas)]
    pb.solarmu, pb.surface_albedo = -1.0, 0.04
    pb.params.transcut = 0.0
    return pb


def gas_absorption_rays_and_truth():
    x = np.linspace(0, 1.0 - 1.0 / 50, 50)
    rays = (x, np.zeros(50), np.full(50, 30.0), np.ones(50), np.zeros(50))
    tau = np.linspace(0.0, 1.0, 50) * 30.0
    return rays, np.exp(-tau) * 0.04 / np.pi * np.exp(-tau)


def thermal_problem(srctype="T", nmu=32, nphi=64):
    """Verify_Thermal / VerifyCombined (tests/test_shdom.py:910-1056 of the
    reference): the same 50x1x11 grid at 11 um with a non-scattering medium
    whose extinction grows linearly in x from 0.001 to 0.5 /km, isothermal at
    288 K, over a Lambertian surface of albedo 0.5 at 300 K, independent-pixel
    mode, no delta-M, a cold (0 K) sky; 'B' adds an overhead sun of flux 1.
    The reference runs NMU=128, NPHI=256; this scene takes the angular
    resolution as arguments (its analytic answer does not depend on it)."""
    pb = brdf_l1_problem()
    ray = pb.species[0]
    npx, npy, npz = ray.extinction.shape
    ray.extinction = np.broadcast_to(np.linspace(0.001, 0.5, npx)[:, None, None], (npx, npy, npz)).astype(np.float32)
    ray.ssalb = np.zeros((npx, npy, npz), np.float32)
    pb.surface_albedo = 0.5
    pb.ground_temperature = 300.0
    pb.temperature = np.full((npx, npy, npz), 288.0, np.float32)
    pb.srctype, pb.units, pb.wavelength = srctype, "R", 11.0
    pb.skyrad = 0.0
    pb.solarmu, pb.solaraz = -1.0, 0.0
    pb.solarflux = 1.0 if srctype == "B" else 0.0
    p = pb.params
    p.num_mu_bins, p.num_phi_bins = nmu, nphi
    p.split_accuracy = p.spherical_harmonics_accuracy = 0.0
    p.solution_accuracy = 1e-5
    p.x_boundary_condition = p.y_boundary_condition = "periodic"
    p.ip_flag, p.tautol, p.deltam = 1, 0.1, False
    return pb


def thermal_rays_and_truth(srctype="T"):
    """Nadir-viewing rays at 30 km and the reference test's closed form: the
    transmitted ground emission, the emission of the isothermal slab, and the
    slab's downwelling flux reflected by the surface (2 E3 written with E1);
    'B' adds the doubly transmitted reflected sun, 0.5 T^2 / pi.  The Planck
    function with physical constants, as the reference test computes it."""
    from scipy.special import exp1

    def planck(t, wl, c=2.99792458e8, h=6.62606876e-34, k=1.3806503e-23):
        wl = wl * 1e-6
        return 2 * h * c ** 2 / wl ** 5 / (np.exp(h * c / (wl * k * t)) - 1.0) * 1e-6

    x = np.linspace(0, 1.0 - 1.0 / 50, 50)
    rays = (x, np.zeros(50), np.full(50, 30.0), np.ones(50), np.zeros(50))
    tau = 30.0 * np.linspace(0.001, 0.5, 50)
    tr = np.exp(-tau)
    b288 = planck(288.0, 11.0)
    rad = 0.5 * planck(300.0, 11.0) * tr + b288 * (1 - tr) + tr * (0.5 * b288 * (-tr * (1 - tau) - tau ** 2 * exp1(tau) + 1))
    if srctype == "B":
        rad = rad + 0.5 * tr * tr / np.pi
    return rays, rad


def thermal_cloud_problem(srctype="T", num_stokes=1, boundary="open", isothermal=None, units="R"):
    """A 16x16x14 absorbing cloud (single-scattering albedo 0.6) in a thin
    Rayleigh layer at 11 um with a temperature that falls with height and
    varies across x, over a 295 K Lambertian ground of albedo 0.05 under a
    200 K sky ('T'; 'B' keeps a zero sky radiance and adds the sun).
    num_stokes=3 uses the polarized mixture phase matrix.  isothermal=T0
    puts the medium, the ground and the sky at T0 K."""
    from at3d_gb300.scenes import cloud_blob, polarized_blob
    if num_stokes == 3:
        pb = polarized_blob(seed=5, nx=16, ny=16, nz=14, dx=0.04, dz=0.06, boundary=boundary, ssa=0.6)
    else:
        pb = cloud_blob(seed=5, nx=16, ny=16, nz=14, dx=0.04, dz=0.06, boundary=boundary)
        pb.species[0].ssalb = np.full_like(pb.species[0].extinction, 0.6)
    npx, npy, npz = pb.shape
    x = np.arange(npx) * pb.delx
    X, _, Z = np.meshgrid(x, np.arange(npy) * pb.dely, pb.zlevels, indexing="ij")
    if isothermal is None:
        pb.temperature = (285.0 + 5.0 * np.cos(2 * np.pi * X / (npx * pb.delx)) - 6.0 * Z).astype(np.float32)
        pb.ground_temperature = 295.0
        pb.skyrad = 200.0 if srctype == "T" else 0.0
    else:
        pb.temperature = np.full((npx, npy, npz), isothermal, np.float32)
        pb.ground_temperature = float(isothermal)
        pb.skyrad = float(isothermal)
    pb.srctype, pb.units, pb.wavelength = srctype, units, 11.0
    if srctype == "T":
        pb.solarflux = 0.0
    pb.surface_albedo = 0.05
    return pb


def brdf_ross_li_problem(lambertian_limit=False):
    """The 50x1x11 Rayleigh scene over the MODIS Ross-Li kernel surface
    ('M': fiso, fgeo, fvol).  lambertian_limit=True sets fgeo = fvol = 0
    and fiso to the albedo ramp of Verify_Lambertian_Surfaces, which makes
    the reflection the Lambertian one of the brdf_L1 golden scene."""
    pb = brdf_l1_problem()
    albedo = np.asarray(pb.surface_albedo, np.float32)
    if lambertian_limit:
        fgeo = fvol = np.zeros((50, 1), np.float32)
        fiso = albedo
    else:
        fiso = np.full((50, 1), 0.12, np.float32)
        fgeo = np.linspace(0.0, 0.04, 50)[:, None].astype(np.float32)
        fvol = np.linspace(0.08, 0.0, 50)[:, None].astype(np.float32)
    pb.surface_brdf = "M"
    pb.surface_params = np.stack([fiso, fgeo, fvol], axis=-1).astype(np.float32)
    pb.surface_albedo = 0.0
    return pb


def thermal_absorbing_blob():
    """A 10x10x8 open-boundary cloud that only absorbs and emits (single-
    scattering albedo 0) in a thin Rayleigh layer, 11 um, temperature
    falling with height and varying across x, 295 K ground, cold sky: the
    gradient case of a thermal source."""
    from at3d_gb300.scenes import cloud_blob
    pb = cloud_blob(seed=4, nx=10, ny=10, nz=8, dx=0.05, dz=0.1, boundary="open")
    pb.species[0].ssalb = np.zeros_like(pb.species[0].extinction)
    npx, npy, _ = pb.shape
    X, _, Z = np.meshgrid(np.arange(npx) * pb.delx, np.arange(npy) * pb.dely, pb.zlevels, indexing="ij")
    pb.temperature = (285.0 + 5 * np.cos(2 * np.pi * X / (npx * pb.delx)) - 6.0 * Z).astype(np.float32)
    pb.srctype, pb.wavelength, pb.solarflux, pb.skyrad, pb.ground_temperature = "T", 11.0, 0.0, 0.0, 295.0
    return pb
