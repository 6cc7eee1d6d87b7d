"""Pins the CPU oracle (oracle/bkma_oracle.c) to golden vectors produced by the
reference's own AdvectionSolver / ConvSolver code (tests/golden/make_golden.py).
Every comparison is bit-exact."""
import numpy as np
import pytest

from oracle import AdvParams


def _params(arr):
    n0, n1, n2, dt, mnx, mxx, mnv, mxv = arr
    return AdvParams(n0=int(n0), n1=int(n1), n2=int(n2), dt=dt, minX=mnx, maxX=mxx,
                     minVx=mnv, maxVx=mxv)


def test_lag_basis_bitexact(oracle, golden):
    for px, coef in zip(golden["lag_px"], golden["lag_coef"]):
        assert np.array_equal(oracle.lag_basis_ref5(float(px)), coef)


def test_lag_basis_partition_of_unity(oracle):
    # the reference basis reproduces constants (its weights sum to 1)
    for px in np.linspace(2.0, 3.0, 33)[:-1]:
        assert abs(oracle.lag_basis_ref5(px).sum() - 1.0) < 1e-14


def test_departure_cells_and_weights_bitexact(oracle, golden):
    cases = golden["stencil_cases"]
    meta, nodes, vals = golden["stencil_meta"], golden["stencil_nodes"], golden["stencil_vals"]
    for (ci, i0, i1), gn, gv in zip(meta, nodes, vals):
        n0, n1, dt, mnx, mxx, mnv, mxv = cases[ci]
        p = AdvParams(n0=int(n0), n1=int(n1), n2=1, dt=dt, minX=mnx, maxX=mxx, minVx=mnv,
                      maxVx=mxv)
        vx = oracle.line_velocity(p, int(i0))
        left, d = oracle.departure(p, int(i1), vx)
        coef = oracle.lag_basis_ref5(d)
        full = np.zeros(int(n1))
        for k in range(6):
            full[(int(n1) + left - 2 + k) % int(n1)] += coef[k]
        nz = np.nonzero(full)[0]
        assert np.array_equal(nz, gn[gn >= 0]), (ci, i0, i1)
        assert np.array_equal(full[nz], gv[: len(nz)]), (ci, i0, i1)


@pytest.mark.parametrize("name", ["small", "odd", "default"])
def test_advection_field_bitexact(oracle, golden, name):
    p = _params(golden[f"adv_{name}_params"])
    cur = golden[f"adv_{name}_init"].copy()
    done = 0
    steps = sorted(int(k.rsplit("step", 1)[1]) for k in golden if k.startswith(f"adv_{name}_step"))
    for s in steps:
        oracle.adv_step(p, cur, s - done)
        done = s
        assert np.array_equal(cur, golden[f"adv_{name}_step{s}"]), (name, s)


@pytest.mark.parametrize("name", ["rand", "wide"])
def test_conv_reference_bitexact(oracle, golden, name):
    n0, C, L, n2, K = (int(v) for v in golden[f"conv_{name}_meta"])
    data = golden[f"conv_{name}_in"].copy()
    oracle.conv_ref_step(data, golden[f"conv_{name}_w"], golden[f"conv_{name}_b"], K, C, L)
    assert np.array_equal(data, golden[f"conv_{name}_out"])


def test_conv_constant_fill(oracle, golden):
    n0, C, L, n2, K = (int(v) for v in golden["conv_const_meta"])
    data = np.full((n0, C * L, n2), 7.3)
    oracle.conv_ref_step(data, np.full((K, C, C), 1.5), np.full(C, 1.0), K, C, L)
    assert np.array_equal(data, golden["conv_const_out"])
    # interior outputs equal 1 + Cin*K*1.5*7.3 (the reference's printed check)
    interior = data[:, 0:L - K + 1, :]  # packed: output iw is point ii1 = iw + K - 1
    assert np.allclose(interior, 1 + C * K * 1.5 * 7.3, rtol=1e-13)


def test_conv_torch_matches_numpy(oracle):
    rng = np.random.default_rng(3)
    B, C, L, K = 2, 5, 37, 4
    x = rng.standard_normal((B, C, L))
    w = rng.standard_normal((6, C, K))
    b = rng.standard_normal(6)
    out = oracle.conv_torch(x, w, b)
    ref = np.zeros((B, 6, L - K + 1))
    for k in range(K):
        ref += np.einsum("oc,bcl->bol", w[:, :, k], x[:, :, k:k + L - K + 1])
    ref += b[None, :, None]
    assert np.allclose(out, ref, rtol=1e-12, atol=1e-12)
    # in place (Cin == Cout): the first L-K+1 columns receive the output
    w2 = rng.standard_normal((C, C, K))
    y = x.copy()
    oracle.conv_torch(y, w2, None, inplace=True)
    want = oracle.conv_torch(x, w2, None)
    assert np.array_equal(y[:, :, :L - K + 1], want)
    assert np.array_equal(y[:, :, L - K + 1:], x[:, :, L - K + 1:])


def test_analytic_validation_zero_iterations(oracle):
    # validation_unittests.cpp:11-31: maxIter = 0 gives exactly 0
    p = AdvParams(n0=5, n1=97, n2=3)
    f = oracle.fill_adv(p)
    assert oracle.validate_adv(p, f, 0) == 0.0


def test_analytic_validation_after_steps(oracle):
    # validation_unittests.cpp:34-94: mean L1 vs sin(4 pi (x - v t)) < 1e-6
    p = AdvParams(n0=16, n1=512, n2=2, dt=1e-4, minVx=0.0, maxVx=1.0)
    f = oracle.fill_adv(p)
    for it in range(1, 11):
        oracle.adv_step(p, f, 1)
        assert oracle.validate_adv(p, f, it) < 1e-6


def test_textbook_lagrange_exact_on_polynomials(oracle):
    for npts in (4, 6, 10):
        px = 0.37 + npts / 2 - 1
        c = oracle.lag_basis_textbook(npts, px)
        for deg in range(npts):
            vals = np.arange(npts, dtype=float) ** deg
            assert abs(c @ vals - px ** deg) < 1e-9 * max(1.0, px ** deg)


def test_uniform_generator_range(oracle):
    u = [oracle.uniform(7, i) for i in range(1000)]
    assert min(u) >= 0.0 and max(u) < 1.0 and abs(np.mean(u) - 0.5) < 0.05
