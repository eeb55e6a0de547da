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


def _phi_float(t, a):
    """Elementary weights Phi(t) of the 13 stages (float64)."""
    v = np.ones(13)
    for ch in t:
        v = v * (a @ _phi_float(ch, a))
    return v


def _gamma(t):
    g = 1 + sum(_size(c) for c in t)
    for c in t:
        g *= _gamma(c)
    return g


def _size(t):
    return 1 + sum(_size(c) for c in t)


def test_dense_output_tables_agree():
    from spectrax_gb300 import tableau
    assert np.array_equal(D.DENSE, np.array(tableau.DENSE))
    for th in (0.0, 0.3, 0.77, 1.0):
        assert np.allclose(D.dense_weights(th), tableau.dense_weights(th), rtol=0, atol=1e-15)


def test_dense_output_order_conditions():
    # order 4 for every rooted tree, order 8 for the tall trees (linear problems),
    # b_j(1) = b_j, b_j(0) = 0 and b_1 = b_2 = 0
    a = D.A
    thetas = np.linspace(0.0, 1.0, 21)
    worst = 0.0
    for q in range(1, 5):
        for t in D.rooted_trees(q):
            p = _phi_float(t, a)
            for th in thetas:
                worst = max(worst, abs(D.dense_weights(th) @ p - th ** q / _gamma(t)))
    tall = ()
    for q in range(1, 9):
        if q > 1:
            tall = (tall,)
        p = _phi_float(tall, a)
        for th in thetas:
            worst = max(worst, abs(D.dense_weights(th) @ p - th ** q / _gamma(tall)))
    assert worst < 1e-12, worst
    assert np.max(np.abs(D.dense_weights(1.0) - D.B)) < 1e-12
    assert np.all(D.dense_weights(0.0) == 0.0)
    assert np.all(D.DENSE[1:3] == 0.0)
    # not order 5 in general: some order-5 tree misses at theta = 1/2
    miss = max(abs(D.dense_weights(0.5) @ _phi_float(t, a) - 0.5 ** 5 / _gamma(t)) for t in D.rooted_trees(5))
    assert miss > 1e-6


def test_interpolated_saves_follow_linear_and_nonlinear_solutions():
    # y' = lam y (linear: the interpolant is 8th order) and y' = y^2 (nonlinear)
    lam = -0.3 + 2.1j
    ts = np.linspace(0.0, 3.0, 61)
    out = D.solve(lambda t, y: lam * y, 0.0, 3.0, np.array([1.0 + 0j]), 0.05, ts=ts,
                  adaptive=True, rtol=1e-10, atol=1e-12)
    assert out["status"] == 0 and out["accepted"] < 40      # steps span several save times
    assert np.max(np.abs(out["ys"][:, 0] - np.exp(lam * ts))) < 1e-9
    ts2 = np.linspace(0.0, 0.9, 46)
    out2 = D.solve(lambda t, y: y * y, 0.0, 0.9, np.array([1.0 + 0j]), 0.01, ts=ts2,
                   adaptive=True, rtol=1e-10, atol=1e-12)
    exact2 = 1.0 / (1.0 - ts2)
    assert np.max(np.abs(out2["ys"][:, 0] - exact2) / exact2) < 5e-8   # order 4 off the linear part
    land = D.solve(lambda t, y: lam * y, 0.0, 3.0, np.array([1.0 + 0j]), 0.05, ts=ts,
                   adaptive=True, rtol=1e-10, atol=1e-12, saveat="land")
    assert land["accepted"] > out["accepted"]                # landing shortens steps
