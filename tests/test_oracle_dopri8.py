"""CPU: the Dopri8 oracle (tableau order conditions, controller behaviour)."""
import numpy as np

from oracle import dopri8 as D


def test_tableau_order_conditions():
    assert [len(D.rooted_trees(q)) for q in range(1, 9)] == [1, 1, 2, 4, 9, 20, 48, 115]
    sol = D.order_condition_residuals(D.B_FR, 8)
    emb = D.order_condition_residuals(D.BHAT_FR, 7)
    assert max(sol.values()) < 1e-16, sol
    assert max(emb.values()) < 1e-16, emb
    # and the pair is exactly 8(7): the next order fails
    assert D.order_condition_residuals(D.B_FR, 9)[9] > 1e-8
    for i, row in D.A_ROWS.items():
        assert abs(float(sum(row.values()) - D.C_FR[i])) < 1e-16


def test_fixed_step_linear_oscillator():
    lam = 1j * 2.0 - 0.1
    f = lambda t, y: lam * y
    out = D.solve(f, 0.0, 2.0, np.array([1.0 + 0j]), 0.05, ts=np.linspace(0, 2, 41), adaptive=False)
    exact = np.exp(lam * out["ts"])
    assert out["status"] == 0 and out["accepted"] == 40
    assert np.max(np.abs(out["ys"][:, 0] - exact)) < 1e-12


def test_adaptive_controller_reaches_tolerance():
    f = lambda t, y: np.array([y[1], -y[0]])
    out = D.solve(f, 0.0, 10.0, np.array([1.0 + 0j, 0j]), 0.01, ts=np.array([10.0]),
                  adaptive=True, rtol=1e-10, atol=1e-12)
    assert out["status"] == 0
    assert abs(out["ys"][-1][0] - np.cos(10.0)) < 1e-9
    assert out["accepted"] > 5


def test_controller_factor_bounds():
    assert D.controller_factor(0.0, True) == 10.0
    assert D.controller_factor(1e-30, True) == 10.0
    assert D.controller_factor(0.9, True) == 1.0
    assert D.controller_factor(1e6, False) == 0.2
    assert abs(D.controller_factor(2.0, False) - 0.9 * 2.0 ** (-1 / 8)) < 1e-15


def test_max_steps_status():
    f = lambda t, y: -y
    out = D.solve(f, 0.0, 1.0, np.array([1.0 + 0j]), 1e-3, adaptive=False, max_steps=10)
    assert out["status"] == 1
