"""Phase-function mixing on the host (no GPU): ``mix_optical_properties``
against a direct restatement of the reference's greedy loop
(phase_function_mixing, src/util.f90:240-348; PHASEFUNC_FROM_WIGNER,
src/shdomsub5.f:2785-2838), the tolerances it promises, and a solve of the
mixture against a solve of the separate species on the oracle (the solver
mixes species exactly, so the difference is the mixing's approximation)."""
import os

import numpy as np
import pytest

from at3d_gb300._abi import Species
from at3d_gb300.medium import (henyey_greenstein_legcoef, hg_matrix_legcoef6, mix_optical_properties,
                               rayleigh_legcoef, rayleigh_legcoef6)


@pytest.fixture(scope="module", autouse=True)
def built():
    from at3d_gb300 import _lib
    from at3d_gb300.build import build
    if not os.path.exists(_lib.LIB):
        build()


def wigner_00_20(x, L):
    d00 = np.zeros(L + 1); d20 = np.zeros(L + 1)
    d00[0] = 1.0
    if L >= 1:
        d00[1] = x
    for l in range(1, L):
        d00[l + 1] = ((2 * l + 1) * x * d00[l] - l * d00[l - 1]) / (l + 1)
    if L >= 2:
        d20[2] = 0.25 * np.sqrt(6.0) * (1 - x * x)
        prev = 0.0
        for l in range(2, L):
            nx = ((2 * l + 1) * x * d20[l] - np.sqrt(l * l - 4.0) * prev) / np.sqrt((l + 1.0) ** 2 - 4.0)
            prev, d20[l + 1] = d20[l], nx
    return d00, d20


def greedy(wig, scat, asym_tol, phase_tol, dolp_tol, nangles):
    """The reference's loop over points (already mixed series wig [npts, L+1, 6])."""
    L = wig.shape[1] - 1
    D = [wigner_00_20(np.cos(np.pi * j / (nangles - 1)), L) for j in range(nangles)]
    d00 = np.array([d[0] for d in D]); d20 = np.array([d[1] for d in D])
    kept, asym, ph, dl = [], [], [], []
    index = np.zeros(len(wig), int)
    f32 = np.float32
    for i, w in enumerate(wig):
        if scat[i] <= 0:
            continue
        a0 = f32(w[1, 0]) / f32(3.0)
        p = (d00 @ w[:, 0].astype(np.float64) / (4 * np.pi)).astype(f32)
        d = (-(d20 @ w[:, 4].astype(np.float64)) / (4 * np.pi)).astype(f32) / p
        use = -1
        if kept:
            errs = [abs(a0 - asym[q]) / asym_tol
                    + np.max(np.abs((p - ph[q]) / np.maximum(f32(0.001), ph[q]))) / phase_tol
                    + np.max(np.abs((d - dl[q]) / np.maximum(f32(0.001), dl[q]))) / dolp_tol for q in range(len(kept))]
            b = int(np.argmin(errs))
            if (abs(a0 - asym[b]) < asym_tol and np.max(np.abs((p - ph[b]) / np.maximum(f32(0.001), ph[b]))) < phase_tol
                    and np.max(np.abs((d - dl[b]) / np.maximum(f32(0.001), dl[b]))) < dolp_tol):
                use = b
        if use < 0:
            kept.append(w); asym.append(a0); ph.append(p); dl.append(d)
            use = len(kept) - 1
        index[i] = use + 1
    return np.array(kept), index


def two_species(seed=0, shape=(6, 5, 4), num_stokes=1):
    rng = np.random.default_rng(seed)
    e1 = rng.uniform(0.0, 10.0, shape).astype(np.float32)
    e2 = rng.uniform(0.0, 2.0, shape).astype(np.float32)
    e1[0, 0, 0] = 0.0; e2[0, 0, 0] = 0.0          # a point without scattering
    if num_stokes == 3:
        hg = np.stack([hg_matrix_legcoef6(g, 0.03, 200) for g in (0.85, 0.7, 0.5)])
        ray = np.zeros((6, 3), np.float32); ray[:, :3] = rayleigh_legcoef6(0.03)
    else:
        hg = np.stack([henyey_greenstein_legcoef(g, 200) for g in (0.85, 0.7, 0.5)])
        ray = rayleigh_legcoef(0.672)
    ti = rng.integers(1, 4, (1,) + shape).astype(np.int32)
    s1 = Species(extinction=e1, ssalb=np.full(shape, 0.99, np.float32), legcoef=hg, table_index=ti,
                 phase_weights=np.ones((1,) + shape, np.float32))
    s2 = Species(extinction=e2, ssalb=np.ones(shape, np.float32), legcoef=ray)
    return s1, s2


@pytest.mark.parametrize("num_stokes", [1, 3])
def test_mixing_matches_restated_greedy_loop(num_stokes):
    s1, s2 = two_species(num_stokes=num_stokes)
    tol = (0.002, 0.01, 0.01)
    mix = mix_optical_properties(s1, s2, asymmetry_tol=tol[0], phase_tol=tol[1], linear_polarization_tol=tol[2],
                                 num_stokes=num_stokes, maxnphase=500)
    shape = s1.extinction.shape
    # the per-point mixtures, x fastest
    def rows(sp):
        lc = np.asarray(sp.legcoef, np.float32)
        if num_stokes == 3:
            lc = lc.reshape(-1, 6, lc.shape[-1]).transpose(0, 2, 1)
        else:
            lc = np.atleast_2d(lc); z = np.zeros(lc.shape + (6,), np.float32); z[..., 0] = lc; lc = z
        return lc
    r1, r2 = rows(s1), rows(s2)
    L = max(r1.shape[1], r2.shape[1])
    pad = lambda r: np.concatenate([r, np.zeros((r.shape[0], L - r.shape[1], 6), np.float32)], 1)
    r1, r2 = pad(r1), pad(r2)
    F = lambda a: np.asarray(a).transpose(2, 1, 0).reshape(-1)
    sc1 = (F(s1.extinction) * F(s1.ssalb)).astype(np.float32)
    sc2 = (F(s2.extinction) * F(s2.ssalb)).astype(np.float32)
    i1 = F(s1.table_index[0])
    wig = (sc1[:, None, None] * r1[i1 - 1] + sc2[:, None, None] * r2[0]).astype(np.float32)
    scat = sc1.astype(np.float64) + sc2
    wig = (wig / np.where(scat > 0, scat, 1)[:, None, None]).astype(np.float32)
    kept, index = greedy(wig, scat, *tol, 180)
    got_index = F(mix.table_index[0])
    want = np.where(index > 0, index, 1)
    assert np.array_equal(got_index, want)
    got = np.asarray(mix.legcoef)
    got = got.transpose(0, 2, 1) if num_stokes == 3 else got[..., None]
    kept = kept.copy(); kept[:, 0, 0] = 1.0
    assert np.allclose(got, kept[..., :got.shape[-1]], rtol=1e-5, atol=1e-7)
    assert len(kept) > 3
    assert np.allclose(mix.extinction, s1.extinction + s2.extinction, rtol=1e-6)
    sca = s1.extinction * s1.ssalb + s2.extinction * s2.ssalb
    ext = s1.extinction + s2.extinction
    assert np.allclose(mix.ssalb, np.where(ext > 0, sca / np.where(ext > 0, ext, 1), 0), rtol=1e-5)
    assert mix.ssalb[0, 0, 0] == 0.0


def test_tolerance_is_met_and_tighter_tolerance_keeps_more():
    s1, s2 = two_species(1)
    loose = mix_optical_properties(s1, s2, asymmetry_tol=0.01, phase_tol=0.05, maxnphase=500)
    tight = mix_optical_properties(s1, s2, asymmetry_tol=0.0005, phase_tol=0.002, maxnphase=500)
    assert np.asarray(tight.legcoef).shape[0] > np.asarray(loose.legcoef).shape[0]
    # every point's entry is within the asymmetry tolerance of its exact mixture
    for mix, atol in ((loose, 0.01), (tight, 0.0005)):
        e1, e2 = s1.extinction * s1.ssalb, s2.extinction * s2.ssalb
        g1 = np.asarray(s1.legcoef)[s1.table_index[0] - 1][..., 1] / 3
        g2 = np.asarray(s2.legcoef)[1] / 3
        g = np.where(e1 + e2 > 0, (e1 * g1 + e2 * g2) / np.where(e1 + e2 > 0, e1 + e2, 1), 0)
        gm = np.asarray(mix.legcoef)[mix.table_index[0] - 1][..., 1] / 3
        m = (e1 + e2) > 0
        assert np.all(np.abs(gm - g)[m] < atol * (1 + 1e-4))


def test_maxnphase_overflow_and_retry():
    s1, s2 = two_species(2)
    with pytest.raises(ValueError, match="Maximum number of phase functions"):
        mix_optical_properties(s1, s2, asymmetry_tol=0.0005, phase_tol=0.002, maxnphase=2)
    ok = mix_optical_properties(s1, s2, asymmetry_tol=0.0005, phase_tol=0.002, maxnphase=2, maxiter=5)
    ref = mix_optical_properties(s1, s2, asymmetry_tol=0.0005, phase_tol=0.002, maxnphase=500)
    assert np.array_equal(ok.table_index, ref.table_index)


def test_mixture_solves_like_the_species(tmp_path):
    """The oracle solves the mixed species and the two separate species;
    the radiances differ by no more than the phase tolerance allows."""
    from at3d_gb300.scenes import cloud_blob, orthographic_views
    from oracle.oracle import Oracle
    import dataclasses
    pb = cloud_blob(seed=3, nx=12, ny=12, nz=10, dx=0.04, dz=0.06, boundary="open")
    cloud, ray = pb.species
    shape = cloud.extinction.shape
    g = np.where(np.arange(shape[0])[:, None, None] < shape[0] // 2, 1, 2) * np.ones(shape, np.int32)
    cloud = dataclasses.replace(cloud, legcoef=np.stack([henyey_greenstein_legcoef(0.85, 64),
                                                         henyey_greenstein_legcoef(0.75, 64)]),
                                table_index=g[None].astype(np.int32), phase_weights=np.ones((1,) + shape, np.float32))
    ray = dataclasses.replace(ray, extinction=np.full(shape, 0.5, np.float32))
    sep = dataclasses.replace(pb, species=[cloud, ray])
    mix = dataclasses.replace(pb, species=[mix_optical_properties(cloud, ray, asymmetry_tol=0.002, phase_tol=0.01,
                                                                  maxiter=5)])
    rays = orthographic_views(pb, 12, 12, zeniths=(0.0, 45.6))
    out = []
    for p in (sep, mix):
        o = Oracle(p)
        o.solve(100)
        out.append(o.render(*rays, nthreads=os.cpu_count() or 1).astype(np.float64))
    rel = np.sqrt(np.mean((out[0] - out[1]) ** 2)) / np.sqrt(np.mean(out[0] ** 2))
    assert rel < 5e-3, rel
