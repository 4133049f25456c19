"""The scene of the reference's Verify_Lambertian_Surfaces test
(tests/test_shdom.py:29-68, :597-632): a 50x1x11 Rayleigh atmosphere at
0.85 um in independent-pixel mode over a variable Lambertian surface, NMU=16,
NPHI=32, solar mu0=-0.707, viewed by 19 upward directions at z=30 km."""
import numpy as np

from at3d_gb300._abi import NumericalParams, Problem, Species
from at3d_gb300.medium import rayleigh_extinction_profile, rayleigh_legcoef


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
