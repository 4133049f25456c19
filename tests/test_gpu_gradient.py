"""GPU Levis gradient (through the C-ABI) against the oracle's restatement,
and the torch.autograd wrapper against the direct adjoint.

Both solvers converge to the same field within the solver tolerance; the
gradients, costs and radiances are compared at relative RMS tolerances
stated per check (the gradient is FP64-accumulated on both sides)."""
import numpy as np
import pytest

from at3d_gb300.scenes import cloud_blob, orthographic_views
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def relrms(a, b):
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-300))


@pytest.fixture(scope="module")
def rte_cls():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from at3d_gb300.solver import RTE
    return RTE


@pytest.mark.parametrize("boundary,npart", [("open", 2), ("periodic", 2)])
def test_levis_gradient_vs_oracle(rte_cls, boundary, npart):
    pb = cloud_blob(seed=6, nx=12, ny=12, nz=10, dx=0.04, dz=0.08, boundary=boundary)
    r = rte_cls.from_problem(pb)
    r.solve(100, verbose=False)
    o = Oracle(pb, fp64=False)
    o.solve(100)
    rays = orthographic_views(pb, 10, 10, zeniths=[0.0, 26.1, -45.6, 60.0])
    base = o.render(*rays, nthreads=8)
    rng = np.random.default_rng(1)
    meas = (base * (1 + 0.05 * rng.standard_normal(base.shape))).astype(np.float32)
    g_gpu, c_gpu, s_gpu = r.levis_gradient(rays, meas, species=0)
    g_orc, c_orc, s_orc = o.levis_gradient(0, rays, meas, nthreads=8)
    g_orc = g_orc.reshape(g_gpu.shape)
    assert relrms(s_gpu, s_orc) < 1e-4
    assert abs(c_gpu - c_orc) <= 2e-3 * abs(c_orc)
    for d in range(2):
        assert relrms(g_gpu[..., d], g_orc[..., d]) < 2e-3, d


def test_autograd_matches_adjoint(rte_cls):
    import torch
    from at3d_gb300.gradient import render_differentiable
    pb = cloud_blob(seed=8, nx=10, ny=10, nz=8, dx=0.05, dz=0.1, boundary="open")
    r = rte_cls.from_problem(pb)
    r.solve(100, verbose=False)
    rays = orthographic_views(pb, 8, 8, zeniths=[0.0, -45.6])
    sp = pb.species[0]
    ext = torch.tensor(np.asarray(sp.extinction, np.float64), requires_grad=True)
    alb = torch.tensor(np.asarray(sp.ssalb, np.float64), requires_grad=True)
    img = render_differentiable(r, ext, alb, rays)
    meas = torch.as_tensor(np.asarray(img.detach().numpy() * 1.1), dtype=img.dtype)
    loss = 0.5 * torch.sum((img - meas) ** 2)
    loss.backward()
    g, cost, _ = r.levis_gradient(rays, meas.numpy().astype(np.float32), species=0)
    assert relrms(ext.grad.numpy(), g[..., 0]) < 1e-5
    assert relrms(alb.grad.numpy(), g[..., 1]) < 1e-5
    assert np.isclose(loss.item(), cost, rtol=1e-5)
