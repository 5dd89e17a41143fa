"""The oracle's optimiser utilities (examples/transformer_optim_utilities.jl):
the OnCell natural cubic spline along the spacing axis, the soft box penalty,
the p-norm and the cost's hard bounds.

The spline is restated from Interpolations.jl's documented meaning of
Cubic(Natural(OnCell())); no golden output of the reference exists for it, so
these tests hold the properties that define it: exact at the knots, zero
second derivative at the cell edges half a step beyond the end knots, linear
data reproduced on the whole domain, and the domain's bounds.
"""
import numpy as np
import pytest

from oracle import bf_oracle as O


def spline(n, seed):
    rng = np.random.default_rng(seed)
    sg = np.linspace(-3e-4, 3e-4, n)
    y = rng.standard_normal((2, 1, n, 2, 2)) + 1j * rng.standard_normal((2, 1, n, 2, 2))
    return sg, y, O.SpacingSpline(y, sg)


def second_derivative_u(sp, r, x):
    """s'' in knot units from the coefficients (piecewise linear in u)."""
    u = 1.0 + (x - sp.first) / sp.step
    i = min(max(int(np.floor(u)), 1), sp.n - 1)
    t = u - i
    c = sp.coef[:, r, 0]
    return (1 - t) * (c[i - 1] - 2 * c[i] + c[i + 1]) + t * (c[i] - 2 * c[i + 1] + c[i + 2])


@pytest.mark.parametrize("n", [2, 3, 5, 9])
def test_spline_exact_at_knots_and_natural_at_cell_edges(n):
    sg, y, sp = spline(n, n)
    for r in range(2):
        for k in range(n):
            assert np.max(np.abs(sp(r, 0, sg[k]) - y[r, 0, k])) < 1e-13
        lo, hi = sp.bounds
        assert np.isclose(lo, sg[0] - 0.5 * (sg[1] - sg[0])) and np.isclose(hi, sg[-1] + 0.5 * (sg[1] - sg[0]))
        assert np.max(np.abs(second_derivative_u(sp, r, lo))) < 1e-12 * np.max(np.abs(y))
        assert np.max(np.abs(second_derivative_u(sp, r, hi))) < 1e-12 * np.max(np.abs(y))


def test_spline_reproduces_linear_data_on_the_whole_domain():
    n = 6
    sg = np.linspace(1e-4, 6e-4, n)
    lin = (0.3 + 2j) * np.arange(n)[None, None, :, None, None] * np.ones((1, 1, n, 2, 2)) + (1 - 1j)
    sp = O.SpacingSpline(lin, sg)
    lo, hi = sp.bounds
    for x in np.linspace(lo, hi, 23):
        u = 1 + (x - sg[0]) / (sg[1] - sg[0])
        assert np.max(np.abs(sp(0, 0, x) - ((0.3 + 2j) * (u - 1) + (1 - 1j)))) < 1e-12
    with pytest.raises(IndexError):
        sp(0, 0, hi + 1e-3 * (sg[1] - sg[0]))


def test_soft_box_penalty_and_p_norm():
    b = (-1.0, 1.0)            # soft depth 0.1: soft bounds -0.9, 0.9
    assert O.soft_box_penalty([0.1, -0.2], b) == 1.0
    assert np.isclose(O.soft_box_penalty([0.95, -0.5], b), 1 - 0.5 ** 6)
    assert np.isclose(O.soft_box_penalty([0.5, 0.45], b), 1 - 0.5 ** 6)     # the sum 0.95 counts
    assert np.isclose(O.soft_box_penalty([-0.95, 0.0], b), 1 - 0.5 ** 6)
    x = np.array([1.0, 2.0, 4.0])
    assert np.isclose(O.p_norm(x, 1), np.mean(x))
    assert O.p_norm(x, -20) < 1.1 and O.p_norm(x, -20) > 1.0                 # ~ min for large negative p
    assert np.isclose(O.p_norm(x, 20), 4.0 * (np.mean((x / 4) ** 20)) ** (1 / 20))


def test_cost_hard_penalty_outside_bounds():
    sg, y, sp = spline(4, 3)
    lo, hi = sp.bounds
    assert O.calc_boostfactor_cost([lo, 0.0], sp, [20e9], None, None, None, None) == 1000.0
    assert O.calc_boostfactor_cost([0.0, hi + 1e-9], sp, [20e9], None, None, None, None) == 1000.0
