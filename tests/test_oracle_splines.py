"""Known-answer tests that pin the oracle's spline restatement.

Port of grid/unit_test/tstSplines.cpp:25-518 (orders 0-6): partition of unity
at three points, stencil indices of a point at a known offset, exact
reproduction of the linear function 4.32 x - 0.31 and of its derivative.
"""
import numpy as np
import pytest

from tests.conftest import float_eq

LOW_X = -3.43
DX = 0.27
RDX = 1.0 / DX


def grid_func(x):
    return 4.32 * x - 0.31


@pytest.mark.parametrize("order", range(7))
def test_partition_of_unity(oracle, order):
    for xp in (-1.4, 2.1789, LOW_X + 5 * DX):
        x0 = oracle.spline_map(order, xp, RDX, LOW_X)
        assert float_eq(oracle.spline_value(order, x0).sum(), 1.0)


@pytest.mark.parametrize("order", range(7))
def test_stencil_and_linear_reproduction(oracle, order):
    # Even orders live on the dual grid: a point a quarter cell past node 4.
    # Odd orders live on the primal grid: a point inside cell 4
    # (tstSplines.cpp:59-60, :117-118, :247-248, :317-318, :392-393).
    if order % 2 == 0:
        anchor = 4
        xp = LOW_X + (anchor + 0.25) * DX
        first = anchor - order // 2
    else:
        anchor = 4
        xp = LOW_X + (anchor + (0.5 if order == 1 else 0.75)) * DX
        first = anchor - (order - 1) // 2
    x0 = oracle.spline_map(order, xp, RDX, LOW_X)
    offsets = oracle.spline_offsets(order)
    stencil = oracle.spline_stencil(order, x0)
    expect = np.arange(first, first + order + 1)
    assert list(int(x0) + offsets) == list(expect)
    assert list(stencil) == list(expect)

    field = np.array([grid_func(LOW_X + s * DX) for s in stencil])
    values = oracle.spline_value(order, x0)
    grads = oracle.spline_gradient(order, x0, RDX)
    if order == 0:
        assert float_eq(field @ values, field[0])
        assert float_eq(field @ grads, 0.0)
    else:
        assert float_eq(field @ values, grid_func(xp))
        assert float_eq(field @ grads, 4.32)


@pytest.mark.parametrize("order", range(1, 7))
def test_gradient_is_derivative_of_value(oracle, order):
    # Central difference of the weights against the analytic gradient.
    rng = np.random.default_rng(order)
    for _ in range(20):
        xp = rng.uniform(0.0, 3.0)
        h = 1e-6
        x_lo = oracle.spline_map(order, xp - h, RDX, LOW_X)
        x_hi = oracle.spline_map(order, xp + h, RDX, LOW_X)
        x0 = oracle.spline_map(order, xp, RDX, LOW_X)
        if int(x_lo) != int(x_hi):
            continue
        fd = (oracle.spline_value(order, x_hi) - oracle.spline_value(order, x_lo)) / (2 * h)
        np.testing.assert_allclose(oracle.spline_gradient(order, x0, RDX), fd, atol=1e-6 * RDX)
