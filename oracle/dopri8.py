"""FP64 Dopri8 stepper with a Diffrax-style step-size controller (test infrastructure only).

Restates the integration that spectrax/_simulation.py:164-180 asks Diffrax for:
``diffeqsolve(ODETerm(ode_system), Dopri8(), PIDController(rtol, atol) | ConstantStepSize(),
t0=0, t1=t_max, dt0=dt, SaveAt(ts=linspace(0, t_max, timesteps)), max_steps=1e6)``.

* Tableau: Prince & Dormand (1981), "High order embedded Runge-Kutta formulae",
  J. Comput. Appl. Math. 7(1):67-75, method RK8(7)13M (13 stages, 8th-order
  solution, 7th-order embedded estimate), the pair Diffrax documents for ``Dopri8``.
  Pinned by its order conditions in ``tests/test_oracle_dopri8.py``.
* Controller: Diffrax's ``PIDController`` defaults (pcoeff=0, icoeff=1, dcoeff=0,
  safety=0.9, factormin=0.2, factormax=10, RMS norm, error order 8): the scaled
  error is rms(e / (atol + rtol*max(|y0|, |y1|))); a step is kept when it is < 1;
  the next step is h*clip(0.9*err**(-1/8), 1 if kept else 0.2, 10).
* Save times, ``saveat="interpolate"`` (default, Diffrax's ``SaveAt(ts)``): steps
  are shortened only to end on t1; a save time t0 < ts <= t0 + h inside an
  accepted step gets y0 + h sum_j b_j(theta) K_j with theta = (ts - t0) / h
  (y1 itself when ts is the step's end).  The weights b_j(theta) are DENSE
  below: a continuous extension of the 13 stages derived for this project from
  the continuous Runge-Kutta order conditions (Hairer, Norsett & Wanner, Solving
  ODEs I, section II.6) -- order 4 for every problem, order 8 for linear
  constant-coefficient problems, b_j(1) = b_j.  Diffrax's own interpolation
  coefficients cannot be run here, so interpolated values are not pinned
  against Diffrax.  ``saveat="land"``: every step is shortened to end exactly on
  the next save time (and on t1); after such a shortened step the next proposal
  is max(h*factor, the proposal before shortening).  The GPU steppers implement
  both modes with the same rules, so GPU and oracle take identical step sequences.
* A rejected step re-uses stage 1 (f at the same (t, y)).
"""
from __future__ import annotations

from fractions import Fraction as Fr

import numpy as np

# ----------------------------------------------------------------- RK8(7)13M tableau
C_FR = [Fr(0), Fr(1, 18), Fr(1, 12), Fr(1, 8), Fr(5, 16), Fr(3, 8), Fr(59, 400), Fr(93, 200),
        Fr(5490023248, 9719169821), Fr(13, 20), Fr(1201146811, 1299019798), Fr(1), Fr(1)]

A_ROWS = {
    1: {0: Fr(1, 18)},
    2: {0: Fr(1, 48), 1: Fr(1, 16)},
    3: {0: Fr(1, 32), 2: Fr(3, 32)},
    4: {0: Fr(5, 16), 2: Fr(-75, 64), 3: Fr(75, 64)},
    5: {0: Fr(3, 80), 3: Fr(3, 16), 4: Fr(3, 20)},
    6: {0: Fr(29443841, 614563906), 3: Fr(77736538, 692538347), 4: Fr(-28693883, 1125000000),
        5: Fr(23124283, 1800000000)},
    7: {0: Fr(16016141, 946692911), 3: Fr(61564180, 158732637), 4: Fr(22789713, 633445777),
        5: Fr(545815736, 2771057229), 6: Fr(-180193667, 1043307555)},
    8: {0: Fr(39632708, 573591083), 3: Fr(-433636366, 683701615), 4: Fr(-421739975, 2616292301),
        5: Fr(100302831, 723423059), 6: Fr(790204164, 839813087), 7: Fr(800635310, 3783071287)},
    9: {0: Fr(246121993, 1340847787), 3: Fr(-37695042795, 15268766246),
        4: Fr(-309121744, 1061227803), 5: Fr(-12992083, 490766935),
        6: Fr(6005943493, 2108947869), 7: Fr(393006217, 1396673457),
        8: Fr(123872331, 1001029789)},
    10: {0: Fr(-1028468189, 846180014), 3: Fr(8478235783, 508512852),
         4: Fr(1311729495, 1432422823), 5: Fr(-10304129995, 1701304382),
         6: Fr(-48777925059, 3047939560), 7: Fr(15336726248, 1032824649),
         8: Fr(-45442868181, 3398467696), 9: Fr(3065993473, 597172653)},
    11: {0: Fr(185892177, 718116043), 3: Fr(-3185094517, 667107341),
         4: Fr(-477755414, 1098053517), 5: Fr(-703635378, 230739211),
         6: Fr(5731566787, 1027545527), 7: Fr(5232866602, 850066563),
         8: Fr(-4093664535, 808688257), 9: Fr(3962137247, 1805957418),
         10: Fr(65686358, 487910083)},
    12: {0: Fr(403863854, 491063109), 3: Fr(-5068492393, 434740067),
         4: Fr(-411421997, 543043805), 5: Fr(652783627, 914296604),
         6: Fr(11173962825, 925320556), 7: Fr(-13158990841, 6184727034),
         8: Fr(3936647629, 1978049680), 9: Fr(-160528059, 685178525),
         10: Fr(248638103, 1413531060)},
}

B_FR = [Fr(14005451, 335480064), Fr(0), Fr(0), Fr(0), Fr(0), Fr(-59238493, 1068277825),
        Fr(181606767, 758867731), Fr(561292985, 797845732), Fr(-1041891430, 1371343529),
        Fr(760417239, 1151165299), Fr(118820643, 751138087), Fr(-528747749, 2220607170),
        Fr(1, 4)]
BHAT_FR = [Fr(13451932, 455176623), Fr(0), Fr(0), Fr(0), Fr(0), Fr(-808719846, 976000145),
           Fr(1757004468, 5645159321), Fr(656045339, 265891186), Fr(-3867574721, 1518517206),
           Fr(465885868, 322736535), Fr(53011238, 667516719), Fr(2, 45), Fr(0)]

STAGES = 13
C = np.array([float(c) for c in C_FR])
A = np.zeros((STAGES, STAGES))
for i, row in A_ROWS.items():
    for j, v in row.items():
        A[i, j] = float(v)
B = np.array([float(b) for b in B_FR])
BHAT = np.array([float(b) for b in BHAT_FR])
E = B - BHAT   # error weights: double difference of the rounded weights (as on the device)

# Dense-output weights: b_j(theta) = sum_k DENSE[j, k] theta^(k+1).  The same
# table as the product's (spectrax_gb300/tableau.py); tests/test_oracle_dopri8.py
# checks both copies against each other and against the continuous order conditions.
DENSE = np.array([
    (1.0225887543186571, -7.670667446945965, 27.66902547999488, -47.67183315927078, 33.46377681416232, -3.361471942445777, 0.26957683985605563, -3.6792478485278544),
    (0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0),
    (0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0),
    (-0.4421091173902579, 26.406870536094136, -184.84492950380366, 374.8074642895895, -187.50765659853084, -73.24848874139202, -61.61212137671032, 106.44097051214344),
    (-0.016770524832150593, 2.735344067839403, -15.823213818196452, 6.754222269863948, 67.35828119490084, -84.62711564401906, -3.1659125143845404, 26.785164968828003),
    (-0.20072361599222294, -8.659354873704325, 72.41722019543212, -165.23218623775102, 90.616848420878, 61.44772288959279, -31.048069957854498, -19.39690914921209),
    (0.47679757022986596, -18.47192139578695, 153.84604554310715, -313.37968335449574, 114.57740262576641, 108.03033023951768, 75.5465634628353, -120.38622188397257),
    (0.35310813749263276, 11.831309677388939, -104.72989197836371, 263.54865955594886, -185.68620659496102, -33.61812083592465, 4.5915511514030305, 44.413101556419335),
    (-0.34706253524185315, -10.277468293537797, 81.19210342937505, -171.80907405747308, 70.61744597042717, 53.04007650498896, 37.04680015843294, -60.222580790785855),
    (0.167271748919783, 4.31464836855168, -31.385871758930698, 56.77008096780195, -5.458949831230438, -28.532677401284158, -22.06850757356576, 26.854568510659924),
    (-0.022168741064052283, -0.32225129840321176, 2.9237861932636586, -8.095256512177215, 6.749080918411023, 0.3572991806069449, -0.4466502168100301, -0.9856520413169936),
    (0.05916230417764668, 0.8225615831834081, -7.362035718957821, 20.157573514806085, -16.46387839878986, -1.0935974138000835, 0.9107258995550841, 2.7313786910726767),
    (-0.05009398061804868, -0.7090709246793181, 6.0977619370794764, -15.849967276842577, 11.733855478966397, 1.6060431641593604, -0.02395587275725969, -2.5545725253080316),
])


def dense_weights(theta):
    """b_j(theta), j = 0..12, by Horner's rule."""
    b = DENSE[:, -1].copy()
    for k in range(DENSE.shape[1] - 2, -1, -1):
        b = b * theta + DENSE[:, k]
    return b * theta


SAFETY, FACTORMIN, FACTORMAX, ERROR_ORDER = 0.9, 0.2, 10.0, 8.0
SNAP = 1e-9   # a step within SNAP*h of the next stop lands on it exactly


def rms_scaled_error(y0, y1, err, rtol, atol):
    """rms(err / (atol + rtol*max(|y0|, |y1|))) over all complex entries."""
    scale = atol + rtol * np.maximum(np.abs(y0), np.abs(y1))
    r = err / scale
    return float(np.sqrt(np.mean(r.real ** 2 + r.imag ** 2)))


def controller_factor(errnorm, accepted):
    """Diffrax PIDController defaults (pure I-controller, error order 8)."""
    if errnorm == 0.0:
        f = FACTORMAX
    elif not np.isfinite(errnorm):
        f = FACTORMIN
    else:
        f = SAFETY * errnorm ** (-1.0 / ERROR_ORDER)
    lo = 1.0 if accepted else FACTORMIN
    return min(max(f, lo), FACTORMAX)


def dopri8_step(f, t, y, h, k1=None, stages=None):
    """One RK8(7)13M step.  Returns (y_new, err, k1); ``stages`` (a list) receives the 13 K_j."""
    ks = [None] * STAGES
    ks[0] = f(t, y) if k1 is None else k1
    for i in range(1, STAGES):
        yi = y.copy()
        for j, a in A_ROWS[i].items():
            yi = yi + (h * float(a)) * ks[j]
        ks[i] = f(t + C[i] * h, yi)
    y_new = y.copy()
    err = np.zeros_like(y)
    for j in range(STAGES):
        if B[j] != 0.0:
            y_new = y_new + (h * B[j]) * ks[j]
        if E[j] != 0.0:
            err = err + (h * E[j]) * ks[j]
    if stages is not None:
        stages[:] = ks
    return y_new, err, ks[0]


def solve(f, t0, t1, y0, dt0, ts=None, adaptive=True, rtol=1e-10, atol=1e-12,
          max_steps=1_000_000, on_save=None, saveat="interpolate"):
    """Integrate y' = f(t, y) from t0 to t1 (``saveat``: "interpolate" or "land").

    Returns dict(ts, ys, accepted, rejected, rhs_evals, status).  ``on_save(i, y)``
    (optional) replaces storing every saved state.
    status: 0 ok, 1 max_steps reached, 2 step size underflow, 3 non-finite state.
    """
    if saveat not in ("interpolate", "land"):
        raise ValueError("saveat must be 'interpolate' or 'land'")
    interp = saveat == "interpolate"
    ts = np.array([t1] if ts is None else ts, dtype=np.float64)
    y = np.array(y0, dtype=np.complex128)
    t = float(t0)
    saved = []
    isave = 0
    def save(i, yy):
        if on_save is None:
            saved.append(yy.copy())
        else:
            on_save(i, yy)
    while isave < len(ts) and ts[isave] <= t:
        save(isave, y)
        isave += 1
    dt = float(dt0)
    k1 = None
    acc = rej = evals = 0
    status = 0
    while t < t1:
        if acc + rej >= max_steps:
            status = 1
            break
        t_stop = min(ts[isave], t1) if (isave < len(ts) and not interp) else t1
        h = dt
        landed = False
        if t + h * (1.0 + SNAP) >= t_stop:
            h = t_stop - t
            landed = True
        if h <= 0.0 or t + h == t:
            status = 2
            break
        evals += STAGES - (1 if k1 is not None else 0)
        ks = []
        y_new, err, k1_now = dopri8_step(f, t, y, h, k1, ks)
        if adaptive:
            en = rms_scaled_error(y, y_new, err, rtol, atol)
            accepted = en < 1.0
            factor = controller_factor(en, accepted)
            dt_next = h * factor
            if accepted and landed and dt_next < dt:
                dt_next = dt
        else:
            accepted = True
            dt_next = dt
        if accepted:
            acc += 1
            t_old, y_old = t, y
            y = y_new
            t = t_stop if landed else t + h
            k1 = None
            if not np.all(np.isfinite(y.view(np.float64))):
                status = 3
                break
            while isave < len(ts) and ts[isave] <= t:
                if interp and ts[isave] != t:
                    w = h * dense_weights((ts[isave] - t_old) / h)
                    yi = y_old.copy()
                    for j in range(STAGES):
                        if DENSE[j].any():
                            yi = yi + w[j] * ks[j]
                    save(isave, yi)
                else:
                    save(isave, y)
                isave += 1
        else:
            rej += 1
            k1 = k1_now
        dt = dt_next
    ys = np.stack(saved) if saved else None
    return dict(ts=ts, ys=ys, accepted=acc, rejected=rej, rhs_evals=evals, status=status, t=t, y=y)


# ----------------------------------------------------------------- order conditions
def rooted_trees(order):
    """All rooted trees with ``order`` nodes, as canonical nested tuples of children."""
    memo = {1: [()]}
    def trees(n):
        if n in memo:
            return memo[n]
        out = set()
        # a tree of n nodes = a root + a multiset of subtrees with total n-1 nodes
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


def order_condition_residuals(b, max_order):
    """max |b . Phi(t) - 1/gamma(t)| per order, in exact rational arithmetic."""
    a = [[A_ROWS.get(i, {}).get(j, Fr(0)) for j in range(STAGES)] for i in range(STAGES)]

    def size(t):
        return 1 + sum(size(c) for c in t)

    def gamma(t):
        g = size(t)
        for c in t:
            g *= gamma(c)
        return g

    cache = {}
    def phi(t):
        if t in cache:
            return cache[t]
        v = [Fr(1)] * STAGES
        for ch in t:
            pc = phi(ch)
            w = [sum(a[i][j] * pc[j] for j in range(STAGES)) for i in range(STAGES)]
            v = [v[i] * w[i] for i in range(STAGES)]
        cache[t] = v
        return v

    res = {}
    for q in range(1, max_order + 1):
        worst = Fr(0)
        for t in rooted_trees(q):
            p = phi(t)
            r = abs(sum(b[i] * p[i] for i in range(STAGES)) - Fr(1, gamma(t)))
            worst = max(worst, r)
        res[q] = float(worst)
    return res
