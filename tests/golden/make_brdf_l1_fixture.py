"""Generates tests/golden/brdf_{L,R,W,D,O}1.npz from the reference's golden files.

Reads the original-SHDOM outputs tests/data/brdf_X1f.out (fluxes) and
tests/data/brdf_X1r.out (radiances) of the reference repository for the
Lambertian (L), RPV (R), wave-Fresnel (W, polarized), Diner (D,
polarized) and 6S ocean (O) surfaces, parsed the way tests/test_shdom.py:17-27 parses them,
and stores the numeric columns.
Run once in a checkout that has the reference mounted:

    python tests/golden/make_brdf_l1_fixture.py /path/to/reference
"""
import os
import sys

import numpy as np


def parse(path, comment="!"):
    rows = []
    with open(path) as f:
        for line in f:
            if comment not in line:
                rows.append(np.array(line.split(), dtype=np.float64))
    return np.array(rows)


def main(ref):
    d = os.path.join(ref, "tests", "data")
    for kind in "LRWDO":
        fl = parse(os.path.join(d, f"brdf_{kind}1f.out"))
        ra = parse(os.path.join(d, f"brdf_{kind}1r.out"))
        out = os.path.join(os.path.dirname(os.path.abspath(__file__)), f"brdf_{kind}1.npz")
        np.savez(out, fluxes=fl, radiances=ra)
        print(out, fl.shape, ra.shape)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_brdf_l1_fixture.py REFERENCE_CHECKOUT")
    main(sys.argv[1])
