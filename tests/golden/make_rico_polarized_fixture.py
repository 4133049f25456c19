"""Builds tests/golden/rico32x36x26w672_pol.npz from the reference's own
polarized verification files (read as text; run once with the path of a reference checkout
as its argument):

* tests/data/rico32x36x26w672.prp -- SHDOM polarized tabulated-phase-function
  property file: NX NY NZ, DELX DELY and the z levels, NUMPHASE, then for
  every phase function the six Wigner-series elements as "K NLEG c_0..c_NLEG",
  then one line "IX IY IZ TEMP EXT ALB IPHASE" per property point;
* tests/data/rico32x36x26w672ar.out -- original SHDOM output of the
  Verify_Solver scene (tests/test_shdom.py:175-261): Stokes I, Q, U at z = 1
  on a 47 x 53 grid of (x, y) for five directions.

The fixture keeps the property grid, the phase-matrix table, the scene
parameters of the output header and the golden I, Q, U.
"""
import os
import sys

import numpy as np

if __name__ == "__main__" and len(sys.argv) != 2:
    sys.exit("usage: make_rico_polarized_fixture.py REFERENCE_CHECKOUT")
REF = sys.argv[1] if len(sys.argv) > 1 else None
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rico32x36x26w672_pol.npz")


def read_prp(path):
    lines = open(path).read().split("\n")
    assert lines[0].startswith("Polarized")
    tok = " ".join(lines[1:]).split()
    pos = 0

    def take(n, conv=float):
        nonlocal pos
        v = [conv(t) for t in tok[pos:pos + n]]
        pos += n
        return v

    npx, npy, npz = take(3, int)
    delx, dely = take(2)
    z = np.array(take(npz), np.float32)
    (numphase,) = take(1, int)
    tables = []
    for _ in range(numphase):
        el = []
        for k in range(6):
            kk, nl = take(2, int)
            assert kk == k + 1
            el.append(np.array(take(nl + 1), np.float64))
        tables.append(el)
    nlmax = max(len(c) for el in tables for c in el)
    leg = np.zeros((numphase, 6, nlmax), np.float32)
    for i, el in enumerate(tables):
        for k, c in enumerate(el):
            leg[i, k, :len(c)] = c
    rest = np.array(tok[pos:], np.float64).reshape(-1, 7)
    ext = np.zeros((npx, npy, npz), np.float32)
    alb = np.zeros((npx, npy, npz), np.float32)
    iph = np.ones((npx, npy, npz), np.int16)
    ix, iy, iz = (rest[:, 0].astype(int) - 1, rest[:, 1].astype(int) - 1, rest[:, 2].astype(int) - 1)
    ext[ix, iy, iz] = rest[:, 4]
    alb[ix, iy, iz] = rest[:, 5]
    iph[ix, iy, iz] = rest[:, 6].astype(np.int16)
    return dict(npx=npx, npy=npy, npz=npz, delx=delx, dely=dely, zlevels=z, legcoef=leg,
                extinction=ext, ssalb=alb, table_index=iph)


def read_out(path):
    rows = []
    for ln in open(path):
        if ln.startswith("!"):
            continue
        v = ln.split()
        if len(v) == 5:
            rows.append([float(t) for t in v])
    return np.array(rows, np.float32)


if __name__ == "__main__":
    d = read_prp(os.path.join(REF, "tests", "data", "rico32x36x26w672.prp"))
    rad = read_out(os.path.join(REF, "tests", "data", "rico32x36x26w672ar.out"))
    # header of the output file: L=7 M=7 NMU=8 NPHI=16, open x and y boundaries
    # (HORIZ_BOUNDARY_COND=3), Lambertian albedo 0.05, SOLAR_MU=-0.5, SOLAR_AZ=0,
    # SPHERICAL_HARMONIC_ACCURACY=0.01, SOLUTION_ACCURACY=1e-4, delta-M,
    # 18 iterations with adaptive splitting at 0.1
    np.savez_compressed(OUT, **d, xy_rows=rad[:, :2], iqu=rad[:, 2:],
                        mu=np.array([1.0, 0.5, 0.2, 0.5, 0.2]), phi_deg=np.array([0.0, 0.0, 0.0, 90.0, 90.0]),
                        nmu=8, nphi=16, solarmu=-0.5, solaraz=0.0, albedo=0.05, shacc=0.01, solacc=1e-4,
                        splitacc=0.1, reference_iterations=18)
    print(OUT, os.path.getsize(OUT), d["legcoef"].shape, rad.shape)
