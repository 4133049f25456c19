"""Thermal emission on the GPU path (srctype 'T' and 'B') against the
oracle, whose own pin is the reference's analytic thermal tests
(tests/test_oracle_thermal.py).  Tolerances as in test_gpu_parity.py:
1e-4 relative RMS on the state after fixed iterations and on converged
radiances."""
import numpy as np
import pytest

from brdf_scene import (brdf_l1_rays, brdf_rpv_problem, brdf_wave_fresnel_problem, thermal_cloud_problem,
                        thermal_problem, thermal_rays_and_truth)
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def relrms(a, b):
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-30))


@pytest.fixture(scope="module")
def rte_cls():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from at3d_gb300.solver import RTE
    return RTE


def _views(pb, n=64):
    xs = np.linspace(0.05, 0.55, n)
    mu = np.where(np.arange(n) % 2 == 0, 1.0, 0.6)
    return xs, np.full(n, 0.3), np.full(n, float(pb.zlevels[-1])), mu, np.full(n, 0.7)


@pytest.mark.parametrize("srctype", ["T", "B"])
def test_thermal_slab(rte_cls, srctype):
    """The reference's Verify_Thermal / VerifyCombined slab at NMU=32,
    NPHI=64 (the GPU's angular limit; the reference runs 128 x 256): the
    GPU render against the oracle at the same resolution, and against the
    closed form within the oracle's own discretisation error plus 1e-4."""
    pb = thermal_problem(srctype, nmu=32, nphi=64)
    r = rte_cls.from_problem(pb)
    r.solve(100, verbose=False)
    o = Oracle(pb)
    o.solve(100)
    rays, truth = thermal_rays_and_truth(srctype)
    got, ref = r.render(*rays), o.render(*rays)
    assert relrms(got, ref) < 1e-4
    assert np.all(np.abs(got - truth) <= np.abs(ref - truth) + 1e-4 * np.abs(truth))


@pytest.mark.parametrize("srctype,boundary", [("T", "open"), ("T", "periodic"), ("B", "open")])
def test_thermal_state_fixed_iterations(rte_cls, srctype, boundary):
    pb = thermal_cloud_problem(srctype, boundary=boundary)
    r = rte_cls.from_problem(pb)
    r.solve(3, verbose=False)
    o = Oracle(pb)
    o.solve(3)
    a, b = r.export_state(), o.export()
    assert np.array_equal(a["ns"], b["ns"])
    assert np.array_equal(a["nr"], b["nr"])
    for k in ("source", "radiance", "fluxes", "dirflux"):
        assert relrms(a[k], b[k]) < 1e-4, k


@pytest.mark.parametrize("srctype,nst", [("T", 1), ("B", 1), ("T", 3)])
def test_thermal_converged_render(rte_cls, srctype, nst):
    pb = thermal_cloud_problem(srctype, num_stokes=nst)
    r = rte_cls.from_problem(pb)
    r.solve(100, verbose=False)
    o = Oracle(pb)
    o.solve(100)
    got, ref = r.render(*_views(pb)), o.render(*_views(pb))
    if nst == 1:
        assert relrms(got, ref) < 1e-4
    else:
        scale = np.sqrt(np.mean(ref[:, 0] ** 2))
        assert relrms(got[:, 0], ref[:, 0]) < 1e-4
        for k in (1, 2):  # Q, U against the I scale
            assert np.sqrt(np.mean((got[:, k] - ref[:, k]) ** 2)) / scale < 1e-4


def test_isothermal_brightness_temperature(rte_cls):
    """Medium, ground and sky at 280 K, units 'T': 280 K in every direction
    (to the 1e-3 the reference's discretisation allows at NMU=8)."""
    pb = thermal_cloud_problem("T", isothermal=280.0, units="T")
    r = rte_cls.from_problem(pb)
    r.solve(100, verbose=False)
    assert np.abs(r.render(*_views(pb)) - 280.0).max() < 0.28


@pytest.mark.parametrize("make", [brdf_rpv_problem, brdf_wave_fresnel_problem], ids=["R", "W"])
def test_thermal_brdf_emission(rte_cls, make):
    """A bidirectional surface emitting with emissivity 1 - R11 (and the
    polarized -R_k1 B terms for the wave-Fresnel surface) under the
    reference's 50x1x11 Rayleigh atmosphere at 288 K, ground at 300 K."""
    pb = make()
    npx, npy, npz = pb.shape
    pb.srctype, pb.wavelength, pb.solarflux, pb.skyrad = "T", 11.0, 0.0, 0.0
    pb.temperature = np.full((npx, npy, npz), 288.0, np.float32)
    pb.ground_temperature = 300.0
    r = rte_cls.from_problem(pb)
    r.solve(100, verbose=False)
    o = Oracle(pb)
    o.solve(100)
    got, ref = r.render(*brdf_l1_rays()), o.render(*brdf_l1_rays())
    if got.ndim == 1:
        assert relrms(got, ref) < 1e-4
    else:
        scale = np.sqrt(np.mean(ref[:, 0] ** 2))
        for k in range(3):
            assert np.sqrt(np.mean((got[:, k] - ref[:, k]) ** 2)) / scale < 1e-4, k


def test_thermal_levis_gradient(rte_cls):
    """The Levis gradient with a thermal source (its emission term) on the
    absorbing cloud: GPU against the oracle after the same 3 iterations
    (the same frozen field up to FP32 rounding), relative RMS 1e-4."""
    from at3d_gb300.scenes import orthographic_views
    from brdf_scene import thermal_absorbing_blob
    pb = thermal_absorbing_blob()
    rays = orthographic_views(pb, 8, 8, zeniths=[0.0, 45.6, -60.0])
    r = rte_cls.from_problem(pb)
    r.solve(3, verbose=False)
    o = Oracle(pb)
    o.solve(3)
    base = o.render(*rays)
    meas = (base * (1 + 0.1 * np.random.default_rng(0).standard_normal(base.shape))).astype(np.float32)
    g_gpu, cost_gpu, _ = r.levis_gradient(rays, meas, 0)
    g_orc, cost_orc, _ = o.levis_gradient(0, rays, meas, nthreads=4)
    g_gpu = np.asarray(g_gpu).reshape(-1, 2)
    for d in range(2):
        assert relrms(g_gpu[:, d], g_orc[:, d]) < 1e-4, d
    assert np.isclose(cost_gpu, cost_orc, rtol=1e-4)

def test_band_units(rte_cls):
    """Units 'B' (the band integral of the Planck function over 800-1000
    cm^-1) on the absorbing cloud, against the oracle."""
    pb = thermal_cloud_problem("T", units="B")
    pb.waveno = (800.0, 1000.0)
    pb.skyrad = 200.0
    r = rte_cls.from_problem(pb)
    r.solve(100, verbose=False)
    o = Oracle(pb)
    o.solve(100)
    assert relrms(r.render(*_views(pb)), o.render(*_views(pb))) < 1e-4
