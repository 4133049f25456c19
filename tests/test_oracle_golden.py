"""Pins the CPU oracle against the reference's own golden vectors.

tests/data/brdf_L1{f,r}.out of the reference (original SHDOM output for the
Verify_Lambertian_Surfaces scene, tests/test_shdom.py:597-632) are stored as
tests/golden/brdf_L1.npz by tests/golden/make_brdf_l1_fixture.py.  The
reference test uses atol 4e-6 (fluxes) and 9e-6 (radiance); the golden files
print five significant digits, so the tolerance here adds half of the last
printed digit of each value.
"""
import numpy as np
import pytest

from brdf_scene import brdf_l1_problem, brdf_l1_rays
from oracle.oracle import Oracle

GOLD = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "brdf_L1.npz"))


def _quantum(v):
    v = np.abs(np.asarray(v, np.float64))
    e = np.floor(np.log10(np.where(v > 0, v, 1.0)))
    return np.where(v > 0, 0.5 * 10.0 ** (e - 4), 5e-7)


@pytest.fixture(scope="module", params=[False, True], ids=["fp32", "fp64"])
def solved(request):
    o = Oracle(brdf_l1_problem(), fp64=request.param)
    iters, solcrit = o.solve(100)
    return o, iters, solcrit


def test_iterations_and_truncation(solved):
    o, iters, solcrit = solved
    assert iters == 3                      # NUMBER_ITERATIONS=3 in brdf_L1r.out
    assert solcrit <= 1e-5
    st = o.export()
    assert int(st["ns"].sum()) == 4050     # NSH=4050 in brdf_L1r.out header


@pytest.mark.parametrize("col,key", [(4, "dirflux"), (3, "down"), (2, "up")])
def test_fluxes(solved, col, key):
    o, _, _ = solved
    st = o.export()
    bot = np.arange(50) * o.sizes["nz"]
    got = {"dirflux": st["dirflux"][bot], "down": st["fluxes"][bot, 0], "up": st["fluxes"][bot, 1]}[key]
    ref = GOLD["fluxes"][:, col]
    assert np.all(np.abs(got - ref) <= 4e-6 + _quantum(ref))


def test_radiances(solved):
    o, _, _ = solved
    got = o.render(*brdf_l1_rays())
    ref = GOLD["radiances"][:, -1]
    assert np.all(np.abs(got - ref) <= 9e-6 + _quantum(ref))
