"""Host logic of bench.py's reference arm: the remaining-iteration estimate
that projects the CPU solves' time comes from each solve's own solution
criteria (a geometric trend), never from the GPU run."""
import numpy as np

import bench


def _solves(crit, solacc):
    cs = bench.CpuSolves.__new__(bench.CpuSolves)
    cs.crit = [list(c) for c in crit]
    cs.solacc = list(solacc)
    return cs


def test_remaining_iterations_follows_the_geometric_trend():
    # criteria falling by 2x per iteration from 1e-1: 1e-4 is reached after log2(1e3) ~ 10 iterations
    c = [0.1 * 0.5 ** k for k in range(4)]
    cs = _solves([c], [1e-4])
    rem = cs.remaining_iterations(0)
    last = c[-1]
    expect = int(np.ceil(np.log(1e-4 / last) / np.log(0.5)))
    assert rem == expect


def test_remaining_iterations_needs_three_points_and_a_falling_trend():
    cs = _solves([[0.1, 0.05], [0.1, 0.2, 0.3, 0.4], [1e-5]], [1e-4, 1e-4, 1e-4])
    assert cs.remaining_iterations(0) is None        # too few criteria for a trend
    assert cs.remaining_iterations(1) is None        # not converging
    assert cs.remaining_iterations(2) == 0           # converged
