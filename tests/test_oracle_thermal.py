"""Thermal emission in the CPU oracle (srctype 'T' and 'B').

Pinned by the reference's own analytic tests Verify_Thermal and
VerifyCombined (tests/test_shdom.py:910-1056): a non-scattering isothermal
slab over an emitting, reflecting Lambertian ground, at the reference's
resolution NMU=128, NPHI=256 and with its check, np.allclose(atol=3e-4)."""
import numpy as np
import pytest

from brdf_scene import thermal_cloud_problem, thermal_problem, thermal_rays_and_truth
from oracle.oracle import Oracle


@pytest.mark.parametrize("srctype", ["T", "B"])
def test_thermal_slab_closed_form(srctype):
    o = Oracle(thermal_problem(srctype, nmu=128, nphi=256))
    o.solve(100)
    rays, truth = thermal_rays_and_truth(srctype)
    got = o.render(*rays)
    assert np.allclose(got, truth, atol=3e-4)


def _views(pb, n=64):
    xs = np.linspace(0.05, 0.55, n)
    mu = np.where(np.arange(n) % 2 == 0, 1.0, 0.6)
    return xs, np.full(n, 0.3), np.full(n, float(pb.zlevels[-1])), mu, np.zeros(n)


@pytest.mark.parametrize("nst", [1, 3])
def test_isothermal_enclosure(nst):
    """Medium, ground and sky at 280 K in brightness-temperature units: the
    radiance is 280 K in every direction and Q = U = 0.  The reference's
    discrete ordinates integrate the hemispheric flux to about 1% at NMU=8
    (the surface reflection term) and its spherical-harmonic source to a
    few 1e-4, so the check is 1e-3 of 280 K."""
    pb = thermal_cloud_problem("T", num_stokes=nst, isothermal=280.0, units="T")
    o = Oracle(pb)
    o.solve(100)
    r = o.render(*_views(pb))
    i = r if nst == 1 else r[:, 0]
    assert np.abs(i - 280.0).max() < 0.28
    if nst == 3:
        assert np.abs(r[:, 1:]).max() < 1e-2


def test_thermal_cloud_fp32_matches_fp64():
    pb = thermal_cloud_problem("T")
    a, b = Oracle(pb), Oracle(pb, fp64=True)
    a.solve(100); b.solve(100)
    ra, rb = a.render(*_views(pb)), b.render(*_views(pb))
    assert np.sqrt(np.mean((ra - rb) ** 2)) / np.sqrt(np.mean(rb ** 2)) < 1e-5


def test_thermal_gradient_matches_frozen_field_differences():
    """The emission term of the Levis source derivative
    (src/polarized/shdomsub4.f:2009-2016): on a cloud that only absorbs and
    emits, the gradient of the L2 cost with respect to the cloud's
    extinction matches central differences of the frozen-field forward
    model within 2% on the interior voxels that carry the most gradient
    (measured: 0.05% to 0.7%)."""
    from at3d_gb300.scenes import orthographic_views
    from brdf_scene import thermal_absorbing_blob
    pb = thermal_absorbing_blob()
    o = Oracle(pb, fp64=True)
    o.solve(100)
    rays = orthographic_views(pb, 8, 8, zeniths=[0.0, 45.6, -60.0])
    base = o.frozen_render(0, 0, 0.0, 0.0, rays)
    meas = (base * (1 + 0.1 * np.random.default_rng(0).standard_normal(base.shape))).astype(np.float32)
    grad, cost, stokes = o.levis_gradient(0, rays, meas, nthreads=4)
    npx, npy, npz = pb.shape
    ext = pb.species[0].extinction.ravel()
    ix, iy = np.unravel_index(np.arange(npx * npy * npz), (npx, npy, npz))[:2]
    interior = (ix > 0) & (ix < npx - 1) & (iy > 0) & (iy < npy - 1)
    order = np.argsort(-np.abs(grad[:, 0]))
    for v in [v for v in order if interior[v]][:4]:
        h = 1e-3 * ext[v]
        pp = o.frozen_render(0, int(v), h, 0.0, rays).astype(np.float64)
        pm = o.frozen_render(0, int(v), -h, 0.0, rays).astype(np.float64)
        fd = (0.5 * np.sum((pp - meas) ** 2) - 0.5 * np.sum((pm - meas) ** 2)) / (2 * h)
        assert abs(grad[v, 0] / fd - 1) < 0.02, (v, grad[v, 0], fd)

def planck_band_shdom(t, w1, w2):
    """Planck's law with SHDOM's constants integrated over [w1, w2] cm^-1
    by adaptive quadrature, W/(m^2 sr)."""
    from scipy.integrate import quad
    c1, c2 = 1.1911e-8, 1.4388  # W/(m^2 sr cm^-4), cm K
    return quad(lambda nu: c1 * nu ** 3 / np.expm1(c2 * nu / t), w1, w2, epsabs=0, epsrel=1e-12)[0]


@pytest.mark.parametrize("band", [(800.0, 1000.0), (20.0, 200.0), (2000.0, 2500.0)])
def test_band_units_black_enclosure(band):
    """Units 'B' (INTEGRATE_PLANCK): a black ground, a black sky
    and the non-scattering slab all at 288 K make every radiance the band
    integral of the Planck function; the bands cover both series of the
    integral (x below and above 1)."""
    pb = thermal_problem("T", nmu=16, nphi=32)
    pb.units, pb.waveno = "B", band
    pb.surface_albedo, pb.ground_temperature = 0.0, 288.0
    pb.skyrad = 288.0
    o = Oracle(pb)
    o.solve(100)
    rays, _ = thermal_rays_and_truth("T")
    got = o.render(*rays)
    # float accumulation along the optically thick columns leaves 1e-5
    assert np.allclose(got, planck_band_shdom(288.0, *band), rtol=2e-5, atol=0)
