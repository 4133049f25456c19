"""RTE.optical_path (at3d/solver.py:793-867; OPTICAL_DEPTH,
src/shdomsub5.f:387-739 of the reference) on the host plan, no GPU: the
extinction integrated along each ray through the base grid, trapezoid per
cell crossing.  Checked where that rule is exact: nadir rays down grid
columns (linear in z within each cell) and slanted rays through a uniform
periodic medium (the path is k H / |mu|)."""
import copy

import numpy as np
import pytest

from at3d_gb300 import scenes
from at3d_gb300.solver import HostPlan, SHDOMError


def _sensor(x, y, z, mu, phi):
    return {"ray_x": np.asarray(x, np.float32), "ray_y": np.asarray(y, np.float32),
            "ray_z": np.asarray(z, np.float32), "ray_mu": np.asarray(mu, np.float64),
            "ray_phi": np.asarray(phi, np.float64)}


def test_nadir_columns_are_trapezoid_sums():
    pb = scenes.cloud_blob(seed=1, nx=10, ny=9, nz=8, dx=0.05, dz=0.08, boundary="open")
    nx, ny, nz = pb.species[0].extinction.shape
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    s = _sensor(ii * pb.delx, jj * pb.dely, np.full(ii.size, 5.0), np.ones(ii.size), np.zeros(ii.size))
    out = HostPlan(pb).optical_path(s)["optical_path"]
    z = np.asarray(pb.zlevels, np.float64)
    ext = sum(np.asarray(sp.extinction, np.float64) for sp in pb.species)
    want = np.trapezoid(ext[ii, jj, :], z, axis=1)
    np.testing.assert_allclose(out, want, rtol=2e-5, atol=1e-7)


def test_uniform_periodic_slant_paths():
    pb = scenes.cloud_blob(seed=1, nx=8, ny=8, nz=7, dx=0.05, dz=0.1, boundary="periodic")
    pb = copy.deepcopy(pb)
    for sp in pb.species:
        sp.extinction = np.full(np.shape(sp.extinction), 2.5 if sp is pb.species[0] else 0.5, np.float32)
    rng = np.random.default_rng(0)
    n = 64
    mu = rng.uniform(0.3, 1.0, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    top = float(np.asarray(pb.zlevels)[-1])
    s = _sensor(rng.uniform(0, 0.4, n), rng.uniform(0, 0.4, n), np.full(n, top), mu, phi)
    out = HostPlan(pb).optical_path(s)["optical_path"]
    h = top - float(np.asarray(pb.zlevels)[0])
    np.testing.assert_allclose(out, 3.0 * h / mu, rtol=2e-5)


def test_deltam_path_and_errors():
    pb = scenes.cloud_blob(seed=1, nx=10, ny=9, nz=8, dx=0.05, dz=0.08, boundary="open")
    x, y, z, mu, phi = scenes.orthographic_views(pb, 5, 5, zeniths=[0.0, 45.6])
    hp = HostPlan(pb)
    s = hp.optical_path(_sensor(x, y, z, mu, phi))
    s = hp.optical_path(s, deltam_scaled_path=True)
    assert np.all(s["optical_path"] > 0)
    assert np.all(s["optical_path_deltam"] <= s["optical_path"] * (1 + 1e-6))
    assert np.any(s["optical_path_deltam"] < 0.9 * s["optical_path"])     # the cloud's forward peak is removed
    up = _sensor([0.1], [0.1], [9.0], [-0.5], [0.0])                       # above the domain, looking up
    assert hp.optical_path(up)["optical_path"][0] == 0.0
    with pytest.raises(SHDOMError, match="below the domain"):
        hp.optical_path(_sensor([0.1], [0.1], [-1.0], [1.0], [0.0]))


def test_net_flux_divergence_conserves_energy():
    """COMPUTE_NETFLUXDIV on a solved state (the oracle's radiance and direct
    beam, the plan's absorption): over a periodic domain the volume integral
    of the net flux divergence equals the net vertical flux (diffuse and
    direct, COMPUTE_SH) through the top less that through the bottom, 2%."""
    from at3d_gb300.solver import compute_netfluxdiv, compute_sh
    from oracle.oracle import Oracle
    pb = scenes.cloud_field(seed=3, nx=16, ny=16, nz=12, dx=0.05, dz=0.05, mean_ext=10.0, boundary="periodic",
                            nmu=8, nphi=16, nleg=128, ssa=0.9, g=0.85)
    hp = HostPlan(pb)
    absorb, emit = hp.point_absorption()
    o = Oracle(pb, fp64=True)
    o.solve(100)
    st = o.export()
    nfd = compute_netfluxdiv(st["radiance"], st["dirflux"], absorb, emit, pb.solarmu, "S")
    nx1, ny1, nz = hp.sizes["nx1"], hp.sizes["ny1"], hp.sizes["nz"]
    nfd = nfd.reshape(nx1, ny1, nz)[:-1, :-1]           # periodic: drop the wrap-around planes
    fz = compute_sh(st["radiance"], st["dirflux"], pb.solarmu, pb.solaraz, "S")[3].reshape(nx1, ny1, nz)[:-1, :-1]
    z = np.asarray(pb.zlevels, np.float64)
    lhs = np.trapezoid(nfd.mean(axis=(0, 1)).astype(np.float64), z)
    rhs = fz[..., -1].mean() - fz[..., 0].mean()
    assert lhs < 0 and rhs < 0
    assert abs(lhs - rhs) <= 0.02 * abs(rhs), (lhs, rhs)
    assert np.all(absorb >= 0) and np.all(emit == 0)


def test_min_optical_path_one_nadir_ray():
    """MIN_OPTICAL_DEPTH: one nadir ray down the middle of a cell column of a
    horizontally uniform medium marks the four corner columns of the cells
    it crosses with the path from the top to each level (the top level with
    the path through the first cell); every other point keeps 999."""
    pb = scenes.cloud_blob(seed=1, nx=6, ny=6, nz=7, dx=0.05, dz=0.1, boundary="periodic")
    pb = copy.deepcopy(pb)
    prof = np.linspace(1.0, 4.0, 7).astype(np.float32)
    pb.species[0].extinction = np.broadcast_to(prof, np.shape(pb.species[0].extinction)).copy()
    pb.species[1].extinction = np.zeros_like(pb.species[1].extinction)
    hp = HostPlan(pb)
    i, j = 2, 3
    s = _sensor([(i + 0.5) * pb.delx], [(j + 0.5) * pb.dely], [5.0], [1.0], [0.0])
    m = hp.min_optical_path(s)
    z = np.asarray(pb.zlevels, np.float64)
    want = np.array([np.trapezoid(prof[k:], z[k:]) for k in range(len(z))])
    want[-1] = want[-2]
    for a in (i, i + 1):
        for b in (j, j + 1):
            np.testing.assert_allclose(m[a, b], want, rtol=2e-5)
    others = np.ones(m.shape[:2], bool)
    others[i:i + 2, j:j + 2] = False
    assert np.all(m[others] == 999.0)
    both = hp.min_optical_path(_sensor([(i + 0.5) * pb.delx] * 2, [(j + 0.5) * pb.dely] * 2, [5.0, 5.0],
                                       [1.0, 1.0], [0.0, 0.0]), do_all=True)
    assert both.shape == (2,) + m.shape and np.array_equal(both[0], m) and np.array_equal(both[1], m)
