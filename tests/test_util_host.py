"""Input formats and helpers on the host (at3d/util.py): the CSV and
2-parameter LWC microphysics files, the Planck function, and phase-matrix
elements from Wigner coefficients against the Rayleigh matrix in closed
form and against the Mie routine's own phase function."""
import os

import numpy as np
import pytest

from at3d_gb300 import util
from at3d_gb300.medium import rayleigh_legcoef6


def test_load_from_csv(tmp_path):
    p = tmp_path / "cloud.txt"
    p.write_text("# a small synthetic cloud\n"
                 "3,2,4      # nx,ny,nz\n"
                 "0.020,0.030   # dx,dy [km, km]\n"
                 "0.5,0.55,0.6,0.7  # altitude levels [km]\n"
                 "x,y,z,lwc,reff\n"
                 "0,0,1,0.1,8.0\n"
                 "2,1,3,0.25,12.5\n")
    d = util.load_from_csv(str(p), density="lwc")
    assert d["density"].shape == (3, 2, 4) and d["density_name"] == "lwc"
    assert d["density"][0, 0, 1] == 0.1 and d["reff"][2, 1, 3] == 12.5
    assert np.isnan(d["reff"][1, 1, 1]) and np.isnan(d["density"]).sum() == 22
    assert np.allclose(d["x"], [0, 0.02, 0.04]) and np.allclose(d["z"], [0.5, 0.55, 0.6, 0.7])
    assert d["dely"] == pytest.approx(0.03)
    with pytest.raises(KeyError):
        util.load_from_csv(str(p), density="iwc")


def test_two_parameter_lwc_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    sc = {"x": np.arange(3) * 0.05, "y": np.arange(2) * 0.05, "z": np.array([0.2, 0.4, 0.6]),
          "density": np.round(rng.uniform(0, 1, (3, 2, 3)), 4), "reff": np.round(rng.uniform(5, 15, (3, 2, 3)), 2)}
    f = tmp_path / "lwc.txt"
    util.to_2parameter_lwc_file(str(f), sc, temperature=[290.0, 288.5, 287.0])
    d = util.load_2parameter_lwc_file(str(f))
    assert np.allclose(d["density"], sc["density"]) and np.allclose(d["reff"], sc["reff"])
    assert np.allclose(d["temperature"], [290.0, 288.5, 287.0]) and np.allclose(d["z"], sc["z"])
    assert d["delx"] == pytest.approx(0.05)


def test_planck_and_frequency():
    # B(10 um, 300 K) = 9.92 W/m^2/um/sr; Wien's law: the peak at 2898/T um
    assert util.planck_function(300.0, 10.0) == pytest.approx(9.92, rel=2e-3)
    lam = np.linspace(5, 20, 3001)
    assert lam[np.argmax(util.planck_function(300.0, lam))] == pytest.approx(2897.8 / 300.0, abs=0.01)
    assert util.freq_to_wavelength(299.792458) == pytest.approx(1000.0)


def test_rayleigh_phase_matrix():
    ang = np.linspace(0, 180, 37)
    mu = np.cos(np.deg2rad(ang))
    P = util.get_phase_function(rayleigh_legcoef6(0.0), ang)
    assert P.shape == (6, 37)
    assert np.allclose(P[0], 0.75 * (1 + mu ** 2))           # P11
    assert np.allclose(P[1], 0.75 * (1 + mu ** 2))           # P22 = P11 for Rayleigh
    assert np.allclose(P[2], 1.5 * mu) and np.allclose(P[3], 1.5 * mu)   # P33, P44
    assert np.allclose(P[4], -0.75 * (1 - mu ** 2))          # P12
    assert np.allclose(P[5], 0.0)                             # P34
    only = util.get_phase_function(rayleigh_legcoef6(0.0)[:1], ang, "P11")
    assert np.allclose(only[0], P[0])
    with pytest.raises(ValueError):
        util.get_phase_function(rayleigh_legcoef6(0.0), ang, ["P13"])


def test_mie_phase_function_normalised():
    from at3d_gb300 import _lib, mie
    from at3d_gb300.build import build
    if not os.path.exists(_lib.LIB):
        build()
    ext, sca, nleg, leg = mie.mie_mono(0.67, 1.33 - 0j, [2.0, 5.0], 200)
    lc = leg / sca[None, None, :]                            # [6, L+1, 2]
    mu, w = np.polynomial.legendre.leggauss(800)
    P = util.get_phase_function(lc, np.rad2deg(np.arccos(mu)), ["P11", "P12"])
    assert P.shape == (2, 800, 2)
    assert np.allclose(0.5 * np.einsum("a,ag->g", w, P[0]), 1.0, atol=1e-5)
    assert np.all(np.abs(P[1]) <= P[0] * (1 + 1e-3) + 1e-3 * P[0].max())
