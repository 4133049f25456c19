"""Makes tests/golden/fp64_cloud_field_128x128x64.npz: radiances of the four
benchmark wavelengths (128x128x64 cloud field, NMU=16/NPHI=32, 64x64
pixels x 9 views) from the oracle run in FP64 for a fixed 30 iterations
(solution accuracy 0, so no early stop).  The GPU transform modes are
compared with it at the same iteration count.  One process per wavelength;
about an hour of CPU time per wavelength.

    python tests/golden/make_fp64_fixture.py [--jobs 4]
"""
import argparse
import os
import sys
from concurrent.futures import ProcessPoolExecutor

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(ROOT, "tests", "golden", "fp64_cloud_field_128x128x64.npz")
NITER = 30


def one(w):
    sys.path.insert(0, ROOT)
    from at3d_gb300.scenes import cloud_field, orthographic_views
    from oracle.oracle import Oracle
    pb = cloud_field(seed=2, wavelength_index=w, nx=128, ny=128, nz=64, solacc=0.0)
    rays = orthographic_views(pb, 64, 64)
    o = Oracle(pb, fp64=True)
    o.init_solution()
    o.solve(NITER)
    return w, np.asarray(o.render(*rays, nthreads=2), np.float64)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=4)
    a = ap.parse_args()
    import multiprocessing as mp
    res = {}
    with ProcessPoolExecutor(a.jobs, mp_context=mp.get_context("spawn")) as ex:
        for w, rad in ex.map(one, range(4)):
            res[f"radiance_{w}"] = rad.astype(np.float32)
            print("wavelength", w, "done", flush=True)
    np.savez_compressed(OUT, iterations=np.int32(NITER), **res)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
