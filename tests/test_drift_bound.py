"""The drift bound of split rows, restated on the CPU.

The screen skips a row when every summation order's FP64 slack is at least
u = fl_ru(U kUMargin), U bounding every |a| (ub - lb) (gdp_device.cuh:
scr_add, scr_slack, scr_skips). A skipped split row keeps the certified margin
m = mn_lo - u - 2^-30 S - 2^-50 |mn_lo| - 2^-80 (scr_margin). Finalize adds
D += fl_ru(|a|_ru fl_ru(lb' - lb + ub - ub')) for every later tightening of one
of its variables, and a marked round leaves the row unread while
fl_ru(D (1 + 2^-22)) <= m (gdp_round.cuh: drift_skips).

These tests restate the screen's FP32 arithmetic and the margin exactly, each
operation rounded in the stated direction, with rational arithmetic. On random
rows they tighten bounds up to the largest drift the rule accepts, and check
the certificate on the tightened row. For every FP64 summation order tried,
each slack is at least u, and every fl(|a| fl(ub - lb)) is at most u. So the
reference's row test skips the row and the row is feasible, exactly as its
screen would decide.
"""
import math
import random
from fractions import Fraction as F

import numpy as np

K_UMARGIN = F(1) + F(1, 2 ** 20)
TINY80 = F(1, 2 ** 80)
INF32 = np.float32(np.inf)


def r32(x: F, mode: str) -> np.float32:
    """x rounded to float32: 'n' nearest-even, 'u' up, 'd' down (normal range)."""
    if x == 0:
        return np.float32(0.0)
    f = np.float32(float(x))
    cands = [np.nextafter(f, -INF32), f, np.nextafter(f, INF32)]
    if mode == "u":
        return min((c for c in cands if F(float(c)) >= x), key=lambda c: F(float(c)))
    if mode == "d":
        return max((c for c in cands if F(float(c)) <= x), key=lambda c: F(float(c)))
    best = min(cands, key=lambda c: (abs(F(float(c)) - x), int(np.float32(c).view(np.int32)) & 1))
    return best


def r64(x: F, mode: str) -> float:
    """x rounded to float64 in the given direction."""
    f = float(x)  # nearest
    if mode == "u" and F(f) < x:
        f = math.nextafter(f, math.inf)
    if mode == "d" and F(f) > x:
        f = math.nextafter(f, -math.inf)
    return f


def screen(a, lb, ub):
    """scr_add over the row: round-to-nearest FP32 copies of coefficients and
    bounds, mn / mx / S / U as the device accumulates them (finite bounds)."""
    mn = mx = S = U = np.float32(0.0)
    for ak, lk, uk in zip(a, lb, ub):
        a32, l32, u32 = np.float32(ak), np.float32(lk), np.float32(uk)
        bmin, bmax = (l32, u32) if a32 > 0 else (u32, l32)
        tmin = r32(F(float(a32)) * F(float(bmin)), "n")
        tmax = r32(F(float(a32)) * F(float(bmax)), "n")
        mn = r32(F(float(mn)) + F(float(tmin)), "n")
        mx = r32(F(float(mx)) + F(float(tmax)), "n")
        s = r32(F(float(abs(tmin))) + F(float(abs(tmax))), "u")
        S = r32(F(float(S)) + F(float(s)), "u")
        d = r32(F(float(u32)) - F(float(l32)), "n")
        w = r32(F(float(abs(u32))) + F(float(abs(l32))), "n")
        inner = r32(F(float(w)) * F(1, 2 ** 21) + F(float(d)), "n")
        U = max(U, r32(F(float(abs(a32))) * F(float(inner)), "n"))
    return mn, mx, S, U


def mag_bracket(x: float):
    """mag_enc: float bracket dn <= |x| <= up (normal range)."""
    m = abs(x)
    dn = r32(F(m), "d")
    return dn, np.nextafter(dn, INF32)


def margin(a, lb, ub, lhs, rhs):
    """(u, m): the screen's certificate value and the certified margin
    (scr_margin); m < 0 when the screen does not skip the row."""
    n = len(a)
    mn, mx, S, U = screen(a, lb, ub)
    k = r32(F(n + 4) * F(0x104, 2 ** 32), "u")  # (n + 4) * 0x1.04p-24, n <= 2^16
    E = r32(F(float(S)) * F(float(k)) + TINY80, "u")
    R = mag_bracket(rhs)
    rhs_dn = -R[1] if rhs < 0 else R[0]
    s_lo = r32(F(float(rhs_dn)) - F(float(r32(F(float(mn)) + F(float(E)), "u"))), "d")
    if lhs == -math.inf:
        lo = s_lo
    else:
        Lh = mag_bracket(lhs)
        lhs_up = -Lh[0] if lhs < 0 else Lh[1]
        t_lo = r32(F(float(r32(F(float(mx)) - F(float(E)), "d"))) - F(float(lhs_up)), "d")
        lo = min(s_lo, t_lo)
    ub_u = r32(F(float(U)) * K_UMARGIN + TINY80, "u")  # scr_u_bound
    u = r32(F(float(ub_u)) * K_UMARGIN, "u")
    if not (u <= lo):
        return u, -1.0
    m = r64(F(float(lo)) - F(float(u)), "d")
    m = r64(F(m) - F(float(S)) * F(1, 2 ** 30), "d")
    m = r64(F(m) - abs(F(float(lo))) * F(1, 2 ** 50), "d")
    return u, r64(F(m) - TINY80, "d")


def drift(a, lb0, ub0, lb1, ub1):
    """D as finalize accumulates it: per changed variable
    fl_ru(|a|_ru32 * fl_ru(fl_ru(lb' - lb) + fl_ru(ub - ub'))), summed in FP64."""
    D = 0.0
    for ak, l0, u0, l1, u1 in zip(a, lb0, ub0, lb1, ub1):
        if l0 == l1 and u0 == u1:
            continue
        dl = r64(F(l1) - F(l0), "u")
        du = r64(F(u0) - F(u1), "u")
        delta = r64(F(dl) + F(du), "u")
        acoef = float(r32(abs(F(ak)), "u"))
        D = D + r64(F(acoef) * F(delta), "u")  # the atomics round to nearest
    return D


def skips(D, m):
    if not math.isfinite(D):  # inf * (1 + 2^-22) <= m and NaN <= m are false on the device
        return False
    return m >= 0 and r64(F(D) * (F(1) + F(1, 2 ** 22)), "u") <= m


def fp64_sum(terms, order):
    s = 0.0
    for k in order:
        s += terms[k]
    return s


def certificate_holds(a, lb, ub, lhs, rhs, u, rng):
    """Every fl(|a| fl(ub - lb)) <= u and, for several FP64 summation orders,
    fl(rhs - minact) >= u and fl(maxact - lhs) >= u."""
    n = len(a)
    d = [abs(ak) * (uk - lk) for ak, lk, uk in zip(a, lb, ub)]
    if max(d) > float(u):
        return False
    tmin = [ak * (lk if ak > 0 else uk) for ak, lk, uk in zip(a, lb, ub)]
    tmax = [ak * (uk if ak > 0 else lk) for ak, lk, uk in zip(a, lb, ub)]
    orders = [list(range(n)), list(range(n - 1, -1, -1))]
    for _ in range(3):
        o = list(range(n))
        rng.shuffle(o)
        orders.append(o)
    for o in orders:
        if rhs - fp64_sum(tmin, o) < float(u):
            return False
        if lhs != -math.inf and fp64_sum(tmax, o) - lhs < float(u):
            return False
    return True


def random_row(rng, n, two_sided):
    a = [rng.choice((-1.0, 1.0)) * math.exp(rng.uniform(math.log(0.1), math.log(10.0))) for _ in range(n)]
    lb = [rng.uniform(-10.0, 0.0) for _ in range(n)]
    ub = [lk + rng.uniform(0.1, 5.0) for lk in lb]
    minact = sum(ak * (lk if ak > 0 else uk) for ak, lk, uk in zip(a, lb, ub))
    maxact = sum(ak * (uk if ak > 0 else lk) for ak, lk, uk in zip(a, lb, ub))
    big = max(abs(ak) * (uk - lk) for ak, lk, uk in zip(a, lb, ub))
    rhs = minact + big * rng.uniform(1.05, 4.0)
    lhs = maxact - big * rng.uniform(1.05, 4.0) if two_sided else -math.inf
    return a, lb, ub, lhs, rhs


def tightened(lb, ub, direction, s):
    """Bounds moved by s along `direction` (non-negative moves of lb up / ub down)."""
    lb1 = [lk + s * dl for lk, (dl, du) in zip(lb, direction)]
    ub1 = [uk - s * du for uk, (dl, du) in zip(ub, direction)]
    return lb1, ub1


def test_drift_within_margin_keeps_the_certificate():
    rng = random.Random(2024)
    checked = 0
    for trial in range(40):
        n = rng.randint(20, 200)
        a, lb, ub, lhs, rhs = random_row(rng, n, two_sided=trial % 2 == 1)
        u, m = margin(a, lb, ub, lhs, rhs)
        if m < 0:
            continue
        # a random tightening direction over a few variables, scaled to the
        # largest step the rule accepts (bisection), then checked at that step
        k = rng.randint(1, max(1, n // 4))
        direction = [(0.0, 0.0)] * n
        for j in rng.sample(range(n), k):
            w = ub[j] - lb[j]
            direction[j] = (rng.uniform(0, 0.4) * w, rng.uniform(0, 0.4) * w)
        lo, hi = 0.0, 1.0
        if skips(drift(a, lb, ub, *tightened(lb, ub, direction, hi)), m):
            lo = hi
        else:
            for _ in range(40):
                mid = 0.5 * (lo + hi)
                if skips(drift(a, lb, ub, *tightened(lb, ub, direction, mid)), m):
                    lo = mid
                else:
                    hi = mid
        if lo == 0.0:
            continue
        lb1, ub1 = tightened(lb, ub, direction, lo)
        assert skips(drift(a, lb, ub, lb1, ub1), m)
        assert certificate_holds(a, lb1, ub1, lhs, rhs, u, rng), (trial, n, lo)
        checked += 1
    assert checked >= 15


def test_infinite_drift_never_skips():
    # an infinite bound that becomes finite makes D infinite
    assert not skips(math.inf, 1.7976931348623157e308)
    assert not skips(float("nan"), 1.0)
    assert not skips(0.0, -1.0)  # the screen did not skip the row: no margin
    assert skips(0.0, 0.0)


def test_margin_is_negative_when_the_screen_cannot_skip():
    rng = random.Random(7)
    for _ in range(10):
        a, lb, ub, lhs, rhs = random_row(rng, 50, two_sided=False)
        big = max(abs(ak) * (uk - lk) for ak, lk, uk in zip(a, lb, ub))
        minact = sum(ak * (lk if ak > 0 else uk) for ak, lk, uk in zip(a, lb, ub))
        # slack below the largest term: the row may tighten, so no certificate
        u, m = margin(a, lb, ub, -math.inf, minact + 0.5 * big)
        assert m < 0
