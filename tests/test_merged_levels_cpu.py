"""The merged-level form of the mixed march's history terms, checked in FP64 on CPU.

The march's right-hand side of step s gets, per level f, G^f W_t(f) - H^f W_u(f)
with the alpha-weighted history combinations of SolverStepLinearT::Solve_Averaging
(SolverStepLinearT.cpp:314-544) and the step's own known load at levels 0/1.  The
tcgen05 engines (march_tc.cu) instead multiply one merged matrix per level, A^f
(the unknown's column of G^f or -H^f, zero for the last dof when its displacement
is prescribed: the state update keeps its prescribed traction, as ExtractField
does), by the unknowns' history, and add the known values' part from three vectors
per level (G^f kt, G^f lt, H^f lu) with per-step coefficients.  This test restates
both sides in numpy and checks that they agree to round-off for random levels,
boundary conditions (a displacement- and traction-prescribed last dof included)
and a load history.
"""
import numpy as np
import pytest


def combine(hist, s, f, lo, hi, a1, a2, a3):
    """The W combination of one level (w_of in march_tc.cu)."""
    w = np.zeros(hist.shape[1])
    m1, m3, m2 = s + 1 - f, s - f, s - 1 - f
    if f >= 2 and lo <= m1 < hi:
        w += a1 * hist[m1]
    if f >= 1 and lo <= m3 < hi:
        w += a3 * hist[m3]
    if lo <= m2 < hi:
        w += a2 * hist[m2]
    if f == 0 and lo <= s - 1 < hi:
        w -= a1 * hist[s - 1]
    return w


def known_coefficients(s, f, a1, a2, a3, amp, c0, c1):
    """(ct, cl, cu) of step s and level f (known_coefficients in march_tc.cu)."""
    ct = cu = 0.0
    for m, w in ((s + 1 - f, a1) if f >= 2 else (None, 0),
                 (s - f, a3) if f >= 1 else (None, 0),
                 (s - 1 - f, a2),
                 (s - 1, -a1) if f == 0 else (None, 0)):
        if m is not None and 1 <= m <= s - 1:
            ct += w * amp[m]
            cu += w
    cl = 0.0
    if f <= 1:
        cf = (1.0 if s == 1 else c0) if f == 0 else (0.0 if s == 1 else c1)
        cl = cf * amp[s]
        cu += cf
    return ct, cl, cu


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_merged_levels_equal_the_g_h_form(seed):
    rng = np.random.default_rng(seed)
    D, L, numstep = 15, 6, 11
    a1, a2 = 0.25, 0.1
    a3 = 1 - a1 - a2
    c0, c1 = 2 * a1 + a3, a1
    G = rng.standard_normal((L, D, D))
    H = rng.standard_normal((L, D, D))
    is_u = rng.random(D) < 0.3
    is_u[D - 1] = True  # the last dof: displacement and traction prescribed
    is_f = ~is_u | (np.arange(D) == D - 1)
    ubc = np.where(is_u, rng.standard_normal(D), 0.0)
    fbc = np.where(is_f, rng.standard_normal(D), 0.0)
    amp = rng.random(numstep + 1) + 0.5

    # histories as the state update writes them (march.cu: k_update_state)
    x = rng.standard_normal((numstep, D))
    u = np.zeros((numstep, D))
    t = np.zeros((numstep, D))
    for m in range(1, numstep):
        u[m] = np.where(is_u, ubc, x[m])
        t[m] = np.where(is_f, fbc * amp[m], 0.0)
        last = np.arange(D) == D - 1
        t[m] = np.where(is_u & ~last, x[m], t[m])

    load_t = np.where(is_f & ~is_u, fbc, 0.0)
    load_u = np.where(is_u, ubc, 0.0)
    # merged form: column selector, A^f, the unknowns' history, the known vectors
    sel = np.where(is_u, np.where(np.arange(D) < D - 1, 1, 0), 2)
    A = np.where(sel == 1, G, np.where(sel == 2, -H, 0.0))
    xh = np.where(sel == 1, t, np.where(sel == 2, u, 0.0))
    kt = np.where(is_f & (~is_u | (np.arange(D) == D - 1)), fbc, 0.0)
    pt, pl, pu = G @ kt, G @ load_t, H @ load_u

    for s in range(1, numstep):
        direct = np.zeros(D)
        merged = np.zeros(D)
        for f in range(min(L - 1, s) + 1):
            wt = combine(t, s, f, 1, s, a1, a2, a3)
            wu = combine(u, s, f, 1, s, a1, a2, a3)
            if f <= 1:  # the step's own known load (k_build_w_old's load terms)
                cf = (1.0 if s == 1 else c0) if f == 0 else (0.0 if s == 1 else c1)
                wt = wt + cf * amp[s] * load_t
                wu = wu + cf * load_u
            direct += G[f] @ wt - H[f] @ wu
            merged += A[f] @ combine(xh, s, f, 1, s, a1, a2, a3)
            ct, cl, cu = known_coefficients(s, f, a1, a2, a3, amp, c0, c1)
            merged += ct * pt[f] + cl * pl[f] - cu * pu[f]
        np.testing.assert_allclose(merged, direct, rtol=0, atol=1e-11 * np.abs(direct).max())


def step_mats(A, nd, a1, a2, a3):
    """B_1 .. B_nd (k_step_mats in march_tc.cu): the weight of the history of step m
    in the right-hand side of step m + d; levels beyond the last are zero."""
    L = A.shape[0]
    lev = lambda f: A[f] if f < L else np.zeros_like(A[0])
    B = [(a2 - a1) * lev(0) + a3 * lev(1) + a1 * lev(2)]
    for d in range(2, nd + 1):
        B.append(a2 * lev(d - 1) + a3 * lev(d) + a1 * lev(d + 1))
    return B


@pytest.mark.parametrize("L", [4, 40])
def test_cross_terms_from_step_distance_matrices(L):
    """The in-block cross terms of the tcgen05 march: the history of steps [a, b)
    into the right-hand sides of steps b .. e - 1, as levels 0 .. e - a with the
    w_of combinations (launch_build_w_merged) and as B_1 .. B_(e-a-1) times the raw
    history (launch_build_w_steps), for every (a, b, e) of the recursive halving of
    32-step blocks; a short level list (L = 4) checks the zero levels past the
    last."""
    rng = np.random.default_rng(7)
    D = 9
    a1, a2 = 0.25, 0.1
    a3 = 1 - a1 - a2
    A = rng.standard_normal((L, D, D))
    x = rng.standard_normal((40, D))
    B = step_mats(A, 31, a1, a2, a3)

    def halves(s0, n, out):
        if n == 1:
            return
        h = n // 2
        halves(s0, h, out)
        out.append((s0, s0 + h, s0 + n))
        halves(s0 + h, n - h, out)

    crosses = []
    halves(1, 32, crosses)
    assert len(crosses) == 31
    for a, b, e in crosses:
        for s in range(b, e):
            levels = np.zeros(D)
            for f in range(min(L - 1, e - a) + 1):
                levels += A[f] @ combine(x, s, f, a, b, a1, a2, a3)
            steps = np.zeros(D)
            for d in range(1, e - a):
                if a <= s - d < b:
                    steps += B[d - 1] @ x[s - d]
            np.testing.assert_allclose(steps, levels, rtol=0,
                                       atol=1e-12 * max(1.0, np.abs(levels).max()))
