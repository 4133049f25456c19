"""The reference's polarized verification scene (Verify_Solver,
tests/test_shdom.py:175-261 of the reference) rebuilt from the committed
fixture tests/golden/rico32x36x26w672_pol.npz: the property grid, the
six-element phase-matrix table and the scene parameters of the original
SHDOM output.  ``rico_problem(split_accuracy=...)``: the original run split
cells adaptively at 0.1 (the fixture's 'splitacc'); 0 keeps the base grid."""
import os

import numpy as np

from at3d_gb300._abi import NumericalParams, Problem, Species

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rico32x36x26w672_pol.npz")


def rico_problem(split_accuracy: float = 0.0):
    g = np.load(FIXTURE)
    sp = Species(extinction=g["extinction"], ssalb=g["ssalb"], legcoef=g["legcoef"],
                 table_index=g["table_index"][None].astype(np.int32),
                 phase_weights=np.ones((1,) + g["extinction"].shape, np.float32))
    prm = NumericalParams(num_mu_bins=int(g["nmu"]), num_phi_bins=int(g["nphi"]),
                          solution_accuracy=float(g["solacc"]), spherical_harmonics_accuracy=float(g["shacc"]),
                          split_accuracy=float(split_accuracy), tautol=0.1, x_boundary_condition="open",
                          y_boundary_condition="open")
    return Problem(delx=float(g["delx"]), dely=float(g["dely"]), zlevels=g["zlevels"], species=[sp],
                   solarmu=float(g["solarmu"]), solaraz=float(g["solaraz"]), solarflux=1.0,
                   surface_albedo=float(g["albedo"]), params=prm, num_stokes=3)


def rico_rays():
    """The golden output's rays: z = 1 km, (x, y) on the 47 x 53 grid of the
    reference test, five directions (mu, phi toward the sensor)."""
    g = np.load(FIXTURE)
    x, y = np.meshgrid(np.arange(0.0, 0.62, 0.0133), np.arange(0.0, 0.70, 0.0133))
    x, y = x.ravel(), y.ravel()
    n = len(g["mu"])
    return (np.tile(x, n), np.tile(y, n), np.ones(x.size * n), np.repeat(g["mu"], x.size),
            np.deg2rad(np.repeat(g["phi_deg"], x.size)))


def rico_golden():
    return np.load(FIXTURE)["iqu"]
