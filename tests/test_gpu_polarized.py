"""GPU parity of the polarized (NSTOKES = 3) path against the polarized
oracle, through the C-ABI.

Tolerances: the Stokes state and radiances after fixed iterations and at
convergence are compared at 1e-4 relative RMS, each Stokes component's RMS
error divided by the RMS of the oracle's I (the radiance scale of the
contract); Q and U are also checked against their own RMS at 1e-3, since
they are one to two orders of magnitude smaller than I.
"""
import copy

import numpy as np
import pytest

from at3d_gb300.medium import hg_matrix_legcoef6
from at3d_gb300.scenes import VIEW_ZENITHS, cloud_blob, orthographic_views, polarized_blob
from oracle.oracle import Oracle
from rico_scene import rico_golden, rico_problem, rico_rays
from test_oracle_polarized import golden_checks

pytestmark = pytest.mark.gpu


def rms(a):
    return float(np.sqrt(np.mean(np.asarray(a, np.float64) ** 2)))


@pytest.fixture(scope="module")
def rte_cls():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from at3d_gb300.solver import RTE
    return RTE


def _scene(**kw):
    return polarized_blob(nx=20, ny=20, nz=14, **kw)


@pytest.mark.parametrize("mode", ["tf32x3", "fp32"])
def test_state_fixed_iterations(rte_cls, mode):
    pb = _scene()
    r = rte_cls.from_problem(pb)
    r.set_transform_mode(mode)
    r.solve(3, verbose=False)
    o = Oracle(pb)
    o.solve(3)
    a, b = r.export_state(), o.export()
    assert a["source"].shape == b["source"].shape == (a["ns"].size, 3, 64)
    assert np.array_equal(a["ns"], b["ns"]) and np.array_equal(a["nr"], b["nr"])
    for key in ("source", "radiance"):
        den = rms(b[key][:, 0])
        for k in range(3):
            assert rms(a[key][:, k] - b[key][:, k]) / den < 1e-4, (key, k)
    assert rms(a["fluxes"] - b["fluxes"]) / rms(b["fluxes"]) < 1e-4


@pytest.mark.parametrize("boundary", ["periodic", "open"])
def test_state_fixed_iterations_stated_size(rte_cls, boundary):
    """The polarized workload at its stated size (64x64x40, NMU 8 / NPHI 16,
    169,000 points on the periodic grid): the Stokes state after 3
    iterations against the oracle, 1e-4 of the RMS of I."""
    pb = polarized_blob(boundary=boundary)
    r = rte_cls.from_problem(pb)
    r.solve(3, verbose=False)
    o = Oracle(pb)
    o.solve(3)
    a, b = r.export_state(), o.export()
    assert np.array_equal(a["ns"], b["ns"]) and np.array_equal(a["nr"], b["nr"])
    for key in ("source", "radiance"):
        den = rms(b[key][:, 0])
        for k in range(3):
            assert rms(a[key][:, k] - b[key][:, k]) / den < 1e-4, (key, k)
    assert rms(a["fluxes"] - b["fluxes"]) / rms(b["fluxes"]) < 1e-4


@pytest.mark.parametrize("mode", ["tf32x3", "fp32"])
def test_converged_render(rte_cls, mode):
    pb = _scene()
    r = rte_cls.from_problem(pb)
    r.set_transform_mode(mode)
    it_g, sc_g = r.solve(100, verbose=False)
    o = Oracle(pb)
    it_o, _ = o.solve(100)
    assert abs(it_g - it_o) <= 1 and sc_g <= pb.params.solution_accuracy
    rays = orthographic_views(pb, 16, 16, VIEW_ZENITHS)
    g = r.render(*rays)
    b = o.render(*rays, nthreads=8)
    assert g.shape == (len(rays[0]), 3)
    den = rms(b[:, 0])
    for k in range(3):
        assert rms(g[:, k] - b[:, k]) / den < 1e-4, k
    for k in (1, 2):
        assert rms(g[:, k] - b[:, k]) / rms(b[:, k]) < 1e-3, k
    sensor = dict(ray_x=rays[0], ray_y=rays[1], ray_z=rays[2], ray_mu=rays[3], ray_phi=rays[4])
    out = r.integrate_to_sensor(sensor)
    assert np.array_equal(out["Q"], g[:, 1]) and np.array_equal(out["U"], g[:, 2])


def test_scalar_limit(rte_cls):
    """b1 = 0 creates no polarization: Q = U = 0 exactly and I equals the
    scalar GPU solve."""
    pb = cloud_blob(nx=16, ny=16, nz=12, dz=0.06)
    pb.species = pb.species[:1]
    p3 = copy.deepcopy(pb)
    p3.num_stokes = 3
    c = hg_matrix_legcoef6(0.85, 0.03, 64)
    c[4] = 0.0
    p3.species[0].legcoef = c
    r1, r3 = rte_cls.from_problem(pb), rte_cls.from_problem(p3)
    r1.solve(100, verbose=False)
    r3.solve(100, verbose=False)
    rays = orthographic_views(pb, 12, 12, VIEW_ZENITHS[:5])
    a, b = r3.render(*rays), r1.render(*rays)
    assert np.all(a[:, 1:] == 0.0)
    assert rms(a[:, 0] - b) / rms(b) < 2e-5


def test_reference_golden_rico(rte_cls):
    """The reference's polarized verification scene: the GPU solve against
    the original SHDOM output (bars of tests/test_oracle_polarized.py, which
    explains the adaptive-splitting difference) and against the oracle."""
    pb = rico_problem()
    r = rte_cls.from_problem(pb)
    it, sc = r.solve(100, verbose=False)
    assert sc <= 1e-4
    rays = rico_rays()
    img = r.render(*rays)
    golden_checks(img, rico_golden())
    o = Oracle(pb)
    o.solve(100)
    b = o.render(*rays, nthreads=8)
    den = rms(b[:, 0])
    for k in range(3):
        assert rms(img[:, k] - b[:, k]) / den < 1e-4, k
