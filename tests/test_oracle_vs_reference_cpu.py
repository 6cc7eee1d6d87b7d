"""The C restatement against the reference's own solvers on random inputs.

Where the reference checkout is present, oracle/build_ref.sh compiles its
AdvectionSolver / ConvSolver sources into oracle/_ref/libbkma_ref.so. The
committed golden vectors pin the restatement at fixed points; these tests
draw seeded random points, parameter sets (negative and large velocities,
shifts of many periods, odd n1, offset domains) and ConvSolver cases, and
require the same bits. Skipped where the reference checkout is absent."""
import os

import numpy as np
import pytest

from oracle import REF_SO, AdvParams, Reference, build_ref


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(REF_SO) and build_ref() is None:
        pytest.skip("the reference checkout is not available here")
    return Reference()


def test_lag_basis_random_points(oracle, ref):
    """AdvectionSolver::lag_basis (src/solvers/AdvectionSolver.hpp:31-51) at
    20000 random points of [2, 3) and at its ends."""
    rng = np.random.default_rng(31)
    pts = np.concatenate([rng.uniform(2.0, 3.0, 20000),
                          [2.0, np.nextafter(3.0, 2.0), np.nextafter(2.0, 3.0), 2.5]])
    for px in pts:
        assert np.array_equal(oracle.lag_basis_ref5(float(px)), ref.lag_basis(float(px))), px


def _adv_params(rng):
    n1 = int(rng.choice([7, 16, 64, 100, 999, 1024]))
    minX = float(rng.choice([0.0, -1.5, 0.25]))
    width = float(rng.choice([1.0, 2.0, 0.3]))
    vmax = float(rng.choice([0.5, 1.0, 7.0, 300.0]))
    vmin = float(rng.choice([-vmax, 0.0, -0.25 * vmax]))
    return AdvParams(n0=int(rng.integers(1, 9)), n1=n1, n2=int(rng.integers(1, 4)),
                     dt=float(rng.choice([1e-4, 1e-3, 0.0371, 0.5])), minX=minX,
                     maxX=minX + width, minVx=vmin, maxVx=vmax)


@pytest.mark.parametrize("seed", range(24))
def test_advection_random_parameter_sets(oracle, ref, seed):
    """AdvectionSolver::operator() under the AdaptiveWg write-back schedule:
    three steps of a random field, bit for bit."""
    rng = np.random.default_rng(1000 + seed)
    p = _adv_params(rng)
    f0 = rng.uniform(-1.0, 1.0, (p.n0, p.n1, p.n2))
    want = ref.adv_step(p, f0.copy(), 3)
    got = oracle.adv_step(p, f0.copy(), 3)
    assert np.array_equal(got, want), p


@pytest.mark.parametrize("seed", range(12))
def test_conv_random_cases(oracle, ref, seed):
    """ConvSolver::operator() (src/solvers/ConvSolver.hpp:20-44) with its
    channel-0 reads, kernel flip and packed outputs, bit for bit."""
    rng = np.random.default_rng(2000 + seed)
    K = int(rng.integers(1, 8))
    C = int(rng.integers(1, 10))
    L = int(rng.integers(K, 40))
    n0, n2 = int(rng.integers(1, 4)), int(rng.integers(1, 4))
    data = rng.uniform(-1.0, 1.0, (n0, C * L, n2))
    w = rng.uniform(-1.0, 1.0, (K, C, C))
    b = rng.uniform(-1.0, 1.0, C)
    want = ref.conv_step(data.copy(), w, b, K, C, L)
    got = oracle.conv_ref_step(data.copy(), w, b, K, C, L)
    assert np.array_equal(got, want), (K, C, L, n0, n2)
