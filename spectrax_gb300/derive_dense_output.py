"""Derive the dense-output (continuous extension) weights of the RK8(7)13M step.

Diffrax answers ``SaveAt(ts=...)`` (spectrax/_simulation.py:175-180) by
evaluating a polynomial interpolant of each accepted step at the save times
instead of shortening steps to land on them.  Diffrax's own Dopri8 interpolant
cannot be inspected or run here, so this module derives one from the published
theory of continuous Runge-Kutta methods (Hairer, Norsett & Wanner, "Solving
Ordinary Differential Equations I", 2nd ed., section II.6; Shampine, "Interpolation
for Runge-Kutta methods", SIAM J. Numer. Anal. 22 (1985) 1014-1027):

    y(t0 + theta h) ~ y0 + h * sum_i b_i(theta) K_i,   b_i(theta) = sum_{j=1..8} beta_ij theta^j,

using only the 13 stage derivatives K_i the step has already computed.  The
weights satisfy, for every theta,

* the continuous order conditions of all rooted trees up to order 4
  (sum_i b_i(theta) Phi_i(t) = theta^rho(t) / gamma(t)); order 5 has no solution
  with these stages (the 17 order-5 conditions exceed the 13-dimensional span);
* the conditions of the tall trees (elementary differentials f'^(q-1) f) up to
  order 8, which make the interpolant 8th-order accurate for linear
  constant-coefficient problems - the streaming, collision and Maxwell parts
  of this right-hand side;
* b_i(1) = b_i, the 8th-order solution weights (continuity at step ends);
* b_1 = b_2 = 0 (0-based stages; the unconstrained optimum has them at ~1e-14,
  so the interpolation reads 11 of the 13 stage vectors).

Of the degree-7 and degree-8 designs tried, this one interpolated a seeded
two-stream trajectory (Nx = 33, Nn = 48, rtol 1e-10) closest to a reference
solution that stops on the save times at rtol 1e-13 (states 1e-14, field energy
3.7e-10 relative).  Any freedom the constraints leave is used to
minimise the integral over theta in [0, 1] of the squared residuals of the
remaining order-5 and order-6 conditions, plus 1e-12 times the squared norm of
the coefficients (which makes the minimiser unique).  The system is solved in 50-digit
arithmetic (mpmath) and rounded to double.  Run as a script to print the table:

    python -m spectrax_gb300.derive_dense_output

The product reads the printed table from ``spectrax_gb300/tableau.py`` and
``csrc/spx_tableau.cuh``; this module is not imported at run time.
"""
from __future__ import annotations

from fractions import Fraction as Fr

DEGREE = 8        # polynomial degree in theta
TALL_ORDER = 8    # tall-tree (linear) order
ORDER = 4         # order for every tree
OBJECTIVE_ORDERS = (5, 6)
RIDGE = 1e-12
ZERO_STAGES = (1, 2)


def _trees(order):
    memo = {1: [()]}

    def trees(n):
        if n in memo:
            return memo[n]
        out = set()

        def parts(rem, max_key, acc):
            if rem == 0:
                out.add(tuple(sorted(acc)))
                return
            for k in range(1, rem + 1):
                for t in trees(k):
                    key = (k, t)
                    if max_key is not None and key > max_key:
                        continue
                    parts(rem - k, key, acc + [t])
        parts(n - 1, None, [])
        memo[n] = sorted(out)
        return memo[n]
    return trees(order)


def _size(t):
    return 1 + sum(_size(c) for c in t)


def _gamma(t):
    g = _size(t)
    for c in t:
        g *= _gamma(c)
    return g


def _tall(q):
    t = ()
    for _ in range(q - 1):
        t = (t,)
    return t


def derive(dps=50):
    """Return beta as a 13 x DEGREE list of mpmath numbers (beta[i][j-1] multiplies theta^j)."""
    import mpmath as mp

    from .tableau import A_FR, B_FR
    mp.mp.dps = dps
    S = 13
    a = [[A_FR.get(i, {}).get(j, Fr(0)) for j in range(S)] for i in range(S)]
    cache = {}

    def phi(t):
        if t in cache:
            return cache[t]
        v = [Fr(1)] * S
        for ch in t:
            pc = phi(ch)
            w = [sum(a[i][j] * pc[j] for j in range(S)) for i in range(S)]
            v = [v[i] * w[i] for i in range(S)]
        cache[t] = v
        return v

    def F(x):
        return mp.mpf(x.numerator) / x.denominator

    d = DEGREE
    n = S * d
    conds = [t for r in range(1, ORDER + 1) for t in _trees(r)]
    conds += [_tall(q) for q in range(ORDER + 1, TALL_ORDER + 1)]
    rows, rhs = [], []
    for t in conds:
        p, r, g = phi(t), _size(t), _gamma(t)
        for j in range(1, d + 1):
            row = [mp.mpf(0)] * n
            for i in range(S):
                row[i * d + j - 1] = F(p[i])
            rows.append(row)
            rhs.append(mp.mpf(1) / g if j == r else mp.mpf(0))
    for i in range(S):
        row = [mp.mpf(0)] * n
        for j in range(1, d + 1):
            row[i * d + j - 1] = mp.mpf(1)
        rows.append(row)
        rhs.append(F(B_FR[i]))
    for i in ZERO_STAGES:
        for j in range(1, d + 1):
            row = [mp.mpf(0)] * n
            row[i * d + j - 1] = mp.mpf(1)
            rows.append(row)
            rhs.append(mp.mpf(0))
    M, bv = mp.matrix(rows), mp.matrix(rhs)
    U, sv, V = mp.svd_r(M, full_matrices=True)
    tol = mp.mpf(10) ** -25
    rank = sum(1 for k in range(len(sv)) if sv[k] > tol)
    # least-squares particular solution (the published tableau's rationals meet
    # the order conditions to ~1e-18 only, so the system is consistent to that level)
    x0 = mp.matrix(n, 1)
    for k in range(rank):
        c = sum(U[i, k] * bv[i] for i in range(M.rows)) / sv[k]
        for i in range(n):
            x0[i] += c * V[k, i]
    null = [[V[k, i] for i in range(n)] for k in range(rank, n)]
    nz = len(null)
    objective = [t for r in OBJECTIVE_ORDERS for t in _trees(r) if t not in conds]
    # residual polynomials sum_j c_j theta^(j+1), j < L; int_0^1 theta^(j+1) theta^(k+1)
    L = max([d] + [_size(t) for t in objective])
    H = mp.matrix(L, L)
    for j in range(L):
        for k in range(L):
            H[j, k] = mp.mpf(1) / (j + k + 3)
    G, gv = mp.matrix(nz, nz), mp.matrix(nz, 1)
    for t in objective:
        r = _size(t)
        pf = [F(v) for v in phi(t)]

        def Pt(vec):
            out = mp.matrix(L, 1)
            for j in range(d):
                out[j] = sum(pf[i] * vec[i * d + j] for i in range(S))
            return out
        e = mp.matrix(L, 1)
        e[r - 1] += mp.mpf(1) / _gamma(t)
        c0 = Pt(x0) - e
        PN = [Pt(null[k]) for k in range(nz)]
        HP = [H * PN[k] for k in range(nz)]
        for k in range(nz):
            gv[k] += sum(HP[k][j] * c0[j] for j in range(L))
            for l in range(k, nz):
                v = sum(HP[k][j] * PN[l][j] for j in range(L))
                G[k, l] += v
                if l != k:
                    G[l, k] += v
    # ridge term RIDGE * |x0 + N z|^2 (the rows of N are orthonormal)
    for k in range(nz):
        G[k, k] += mp.mpf(RIDGE)
        gv[k] += mp.mpf(RIDGE) * sum(null[k][i] * x0[i] for i in range(n))
    x = x0.copy()
    if nz:
        z = mp.lu_solve(G, -gv)
        for k in range(nz):
            for i in range(n):
                x[i] += z[k] * null[k][i]
    beta = [[x[i * d + j] for j in range(d)] for i in range(S)]
    for i in ZERO_STAGES:
        beta[i] = [mp.mpf(0)] * d
    return beta


def main():
    beta = derive()
    print("# DENSE[i][j]: coefficient of theta^(j+1) in b_i(theta)")
    for row in beta:
        print("    (" + ", ".join(repr(float(v)) for v in row) + "),")


if __name__ == "__main__":
    main()
