"""The oracle's restatement of the Levis approximate gradient
(LEVISAPPROX_GRADIENT, adjoint branch, src/polarized/shdomsub4.f:288-809)
against central differences of the forward model it approximates: render
with one voxel's extinction or albedo changed, the medium, direct beam and
source function recomputed from the frozen radiance field.

The Levis gradient is the reference's approximation (it is not the exact
derivative of this forward model either: e.g. the subgrid step count and
the source truncation are held fixed), so the check is on the voxels that
carry most of the gradient, at a few percent."""
import numpy as np
import pytest

from at3d_gb300.scenes import cloud_blob, orthographic_views
from oracle.oracle import Oracle


@pytest.fixture(scope="module")
def solved():
    pb = cloud_blob(seed=4, nx=10, ny=10, nz=8, dx=0.05, dz=0.1, boundary="open")
    o = Oracle(pb, fp64=True)
    o.solve(100)
    rays = orthographic_views(pb, 8, 8, zeniths=[0.0, 45.6, -60.0])
    base = o.frozen_render(0, 0, 0.0, 0.0, rays)
    rng = np.random.default_rng(0)
    meas = (base * (1 + 0.1 * rng.standard_normal(base.shape))).astype(np.float32)
    grad, cost, stokes = o.levis_gradient(0, rays, meas, nthreads=4)
    return pb, o, rays, meas, grad, cost, stokes, base


def test_cost_is_half_squared_residual(solved):
    pb, o, rays, meas, grad, cost, stokes, base = solved
    assert np.isclose(cost, 0.5 * np.sum((stokes.astype(np.float64) - meas) ** 2), rtol=1e-9)
    assert np.sqrt(np.mean((stokes - base) ** 2)) / np.sqrt(np.mean(base ** 2)) < 2e-4


def _fd(o, pb, rays, meas, v, idr):
    ext = pb.species[0].extinction.ravel()
    alb = pb.species[0].ssalb.ravel()
    h = 1e-3 * (ext[v] if idr == 0 else alb[v])
    if idr == 1 and alb[v] + h > 1:
        h = -h
    d = (h, 0.0) if idr == 0 else (0.0, h)
    pp = o.frozen_render(0, int(v), d[0], d[1], rays).astype(np.float64)
    pm = o.frozen_render(0, int(v), -d[0], -d[1], rays).astype(np.float64)
    return (0.5 * np.sum((pp - meas) ** 2) - 0.5 * np.sum((pm - meas) ** 2)) / (2 * h)


# Interior voxels (not on the open-boundary edge columns, whose edge-cell
# traces the approximation handles more coarsely): 2% on extinction, 1% on
# albedo; edge-column voxels: 15%.
@pytest.mark.parametrize("idr,tol", [(0, 0.02), (1, 0.01)])
def test_matches_frozen_field_differences(solved, idr, tol):
    pb, o, rays, meas, grad, cost, stokes, base = solved
    nx, ny, nz = pb.species[0].extinction.shape
    ix, iy = np.unravel_index(np.arange(nx * ny * nz), (nx, ny, nz))[:2]
    interior = (ix > 0) & (ix < nx - 1) & (iy > 0) & (iy < ny - 1)
    order = np.argsort(-np.abs(grad[:, idr]))
    for v in [v for v in order if interior[v]][:4]:
        fd = _fd(o, pb, rays, meas, v, idr)
        assert abs(grad[v, idr] - fd) <= tol * abs(fd), (v, grad[v, idr], fd)
    for v in [v for v in order if not interior[v]][:3]:
        fd = _fd(o, pb, rays, meas, v, idr)
        assert abs(grad[v, idr] - fd) <= 0.15 * abs(fd), (v, grad[v, idr], fd)


def test_phase_derivative_matches_frozen_field_differences(solved):
    """The third unknown of LEVISAPPROX_GRADIENT: the phase function moved
    along a derivative series (DLEG / DIPHASEP; here d/dg of the cloud's
    Henyey-Greenstein series, with delta-M, so the DFP terms of
    PREPARE_DERIV_INTERPS and the DSINGSCAT term enter).  Against central
    differences of the frozen-field forward model with that voxel's phase
    function moved, 1% on the five voxels that carry most of the gradient;
    the extinction and albedo columns are those of the two-unknown pass."""
    pb, o, rays, meas, grad, cost, stokes, base = solved
    nleg = pb.species[0].legcoef.shape[-1]
    l = np.arange(nleg)
    dleg = ((2 * l + 1) * l * 0.85 ** np.maximum(l - 1, 0)).astype(np.float32)
    ng = pb.species[0].extinction.size
    w = np.random.default_rng(1).standard_normal(len(rays[0]))
    before = o.render(*rays)
    G = o.levis_adjoint_phase(0, rays, w, dleg[None], np.ones((ng, 1), np.int32), nthreads=4)
    assert np.array_equal(G[:, :2], o.levis_adjoint(0, rays, w, nthreads=4).reshape(-1, 2))
    for v in np.argsort(-np.abs(G[:, 2]))[:5]:
        h = 1e-3
        pp = o.frozen_render_phase(0, int(v), h, dleg, rays).astype(np.float64)
        pm = o.frozen_render_phase(0, int(v), -h, dleg, rays).astype(np.float64)
        fd = np.dot(w, pp - pm) / (2 * h)
        assert abs(G[v, 2] - fd) <= 0.01 * abs(fd), (v, G[v, 2], fd)
    assert np.array_equal(o.render(*rays), before)      # the perturbed renders leave the solver as it was


def test_effective_radius_gradient_chain():
    """An effective-radius derivative end to end on the oracle: the
    generator's derivatives of extinction, albedo and phase mixture with
    respect to reff (reff tabulated, multilinear phase weights) combined
    with the three unknowns of the Levis gradient equal the central
    differences of the frozen-field model along the same direction (2% on
    the voxels that carry most of the gradient)."""
    from at3d_gb300 import mie, size_distribution as sd
    from at3d_gb300._abi import NumericalParams, Problem, Species
    from at3d_gb300.medium import OpticalPropertyGenerator, rayleigh_legcoef
    from at3d_gb300.scenes import mie_microphysics
    import os
    from at3d_gb300 import _lib
    from at3d_gb300.build import build
    if not os.path.exists(_lib.LIB):
        build()
    mono = {0.672: mie.get_mono_table("Water", (0.672, 0.672), minimum_effective_radius=4.0,
                                      max_integration_radius=16.0, refractive_index=1.331 - 1.6e-8j, verbose=False)}
    gen = OpticalPropertyGenerator("cloud", mono, sd.gamma, maxnphase=6, interpolation_mode="exact",
                                   reff={"coord_min": 4.0, "coord_max": 14.0, "npoints": 6, "spacing": "linear"},
                                   veff=np.array([0.1]))
    micro = mie_microphysics(seed=3, nx=8, ny=8, nz=8, dx=0.05, dz=0.08, peak=0.3, reff=(5.3, 12.7))
    micro["veff"] = np.full(micro["density"].shape, 0.1)
    cloud = gen(micro)[0.672]
    assert cloud.table_index.shape[0] == 2          # reff tabulated with linear phase weights
    der = gen.calculate_derivatives(["reff"], micro)[0.672]["reff"]
    shape = micro["density"].shape
    ray = Species(extinction=np.full(shape, 0.01, np.float32), ssalb=np.ones(shape, np.float32),
                  legcoef=rayleigh_legcoef(0.672))
    params = NumericalParams(num_mu_bins=8, num_phi_bins=16, solution_accuracy=1e-5, split_accuracy=0.0,
                             x_boundary_condition="open", y_boundary_condition="open")
    pb = Problem(delx=0.05, dely=0.05, zlevels=(np.arange(8) * 0.08).astype(np.float32), species=[cloud, ray],
                 solarmu=-float(np.cos(np.deg2rad(30.0))), solaraz=0.0, params=params, surface_albedo=0.05)
    o = Oracle(pb, fp64=True)
    o.solve(100)
    rays = orthographic_views(pb, 8, 8, zeniths=[0.0, 45.6, -60.0])
    w = np.random.default_rng(2).standard_normal(len(rays[0]))
    ng = int(np.prod(shape))
    dleg = der["legcoef"].reshape(ng, -1).astype(np.float32)
    diph = np.repeat(np.arange(1, ng + 1, dtype=np.int32)[:, None], 2, axis=1)
    G = o.levis_adjoint_phase(0, rays, w, dleg, diph, nthreads=4)
    dext, dalb = der["extinction"].reshape(-1), der["ssalb"].reshape(-1)
    dreff = G[:, 0] * dext + G[:, 1] * dalb + G[:, 2]
    for v in np.argsort(-np.abs(dreff))[:5]:
        h = 1e-2
        pp = o.frozen_render_phase(0, int(v), h, dleg[v], rays, dext=h * dext[v], dalb=h * dalb[v])
        pm = o.frozen_render_phase(0, int(v), -h, dleg[v], rays, dext=-h * dext[v], dalb=-h * dalb[v])
        fd = np.dot(w, pp.astype(np.float64) - pm) / (2 * h)
        assert abs(dreff[v] - fd) <= 0.02 * abs(fd), (v, dreff[v], fd)
