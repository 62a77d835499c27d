"""The planner's fast rejection prunes only pairs its full bound prunes too.

plan.cu tests each (query, list) pair first with fast_reject (float products
with a 2^-16 margin on every step, no square root) and only the pairs that
test keeps with prune_threshold (directed-rounding products and square
roots); a pair is pruned when its threshold exceeds the query's tau.  Both
are restated here with exact rational arithmetic for the rounding of every
float operation (down, up or to nearest, as the kernel's intrinsics and its
default operations round), with the plan constants as fill_plan_args makes
them, and checked on seeded random pairs and on pairs placed just past the
fast test's limit, for both metrics: whenever D(q, r) exceeds the fast limit,
prune_threshold must exceed tau.  The fast test's one fused step (the query
term's product and sum) is checked both fused and rounded twice.
"""
import math
import random
from fractions import Fraction as Fr

import numpy as np
import pytest

F32_MAX = Fr(float(np.finfo(np.float32).max))
MARGIN = Fr(1) + Fr(1, 2 ** 16)


def _up(v):
    return np.nextafter(np.float32(v), np.float32(np.inf), dtype=np.float32)


def _down(v):
    return np.nextafter(np.float32(v), np.float32(-np.inf), dtype=np.float32)


def rd(x):
    """Largest float32 <= x (x a Fraction, non-negative here)."""
    if x > F32_MAX:
        return np.float32(np.finfo(np.float32).max)
    v = np.float32(float(x))
    while Fr(float(v)) > x:
        v = _down(v)
    while np.isfinite(_up(v)) and Fr(float(_up(v))) <= x:
        v = _up(v)
    return v


def ru(x):
    """Smallest float32 >= x (+inf past the largest float)."""
    if x > F32_MAX:
        return np.float32(np.inf)
    v = np.float32(float(x))
    while Fr(float(v)) < x:
        v = _up(v)
        if not np.isfinite(v):
            return v
    while Fr(float(_down(v))) >= x:
        v = _down(v)
    return v


def rn(x):
    """Nearest float32, ties to even (+inf past the overflow threshold)."""
    lo, hi = rd(x), ru(x)
    if lo == hi:
        return lo
    if not np.isfinite(hi):
        limit = F32_MAX + (F32_MAX - Fr(float(_down(np.float32(np.finfo(np.float32).max))))) / 2
        return hi if x >= limit else lo
    dl, dh = x - Fr(float(lo)), Fr(float(hi)) - x
    if dl != dh:
        return lo if dl < dh else hi
    return lo if int(np.float32(lo).view(np.uint32)) % 2 == 0 else hi


def fr(v):
    return Fr(float(v)) if np.isfinite(v) else None


def mul(a, b, r):
    if not (np.isfinite(a) and np.isfinite(b)):
        return np.float32(np.inf)
    return r(fr(a) * fr(b))


def div(a, b, r):
    if not np.isfinite(a):
        return np.float32(np.inf)
    return r(fr(a) / fr(b))


def add(a, b, r):
    if not (np.isfinite(a) and np.isfinite(b)):
        return np.float32(np.inf)
    return r(fr(a) + fr(b))


def sub(a, b, r):
    return r(fr(a) - fr(b))


def sqrt_rd(a):
    v = np.float32(math.sqrt(float(a)))
    x = fr(a)
    while Fr(float(v)) ** 2 > x:
        v = _down(v)
    while Fr(float(_up(v))) ** 2 <= x:
        v = _up(v)
    return v


def sqrt_ru(a):
    if not np.isfinite(a):
        return np.float32(np.inf)
    v = np.float32(math.sqrt(float(a)))
    x = fr(a)
    while Fr(float(v)) ** 2 < x:
        v = _up(v)
    while v > 0 and Fr(float(_down(v))) ** 2 >= x:
        v = _down(v)
    return v


class Plan:
    """fill_plan_args' constants (engine.cu) for padded dimension dp."""

    def __init__(self, dp, l1):
        g = (dp + 8) * 1.1920928955078125e-07
        self.l1 = l1
        self.opg_ru = ru(Fr(1.0 + g))
        self.omg_rd = rd(Fr(1.0 - g))
        self.c_ru = ru(Fr(1.0 + 3.0 * g))
        self.opc_ru = ru(Fr(2.0 + 3.0 * g))
        self.inv_opg_rd = rd(Fr(1.0 / (1.0 + g) * (1.0 - 2.0 ** -50)))
        self.inv_omg_ru = ru(Fr(1.0 / (1.0 - g) * (1.0 + 2.0 ** -50)))
        self.inv_opc_rd = rd(Fr(1.0 / (2.0 + 3.0 * g) * (1.0 - 2.0 ** -50)))

    def query_term(self, dq0):
        t = mul(dq0, self.inv_omg_ru, ru)
        return mul(self.c_ru, t if self.l1 else sqrt_ru(t), ru)

    def psi_bound(self, psi):
        t = div(psi, self.omg_rd, ru)
        return t if self.l1 else sqrt_ru(t)

    def prune_threshold(self, dqr, chi0, hpsi):
        t = mul(dqr, self.inv_opg_rd, rd)
        lo = t if self.l1 else sqrt_rd(t)
        lb1 = sub(lo, hpsi, rd) if np.isfinite(hpsi) else np.float32(-np.inf)
        num = sub(lo, chi0, rd) if np.isfinite(chi0) else np.float32(-np.inf)
        lb2 = mul(num, self.inv_opc_rd, rd) if num > 0 else np.float32(0)
        lb = max(lb1, lb2)
        if not lb > 0:
            return np.float32(0)
        return mul(lb, self.omg_rd, rd) if self.l1 else mul(mul(lb, lb, rd), self.omg_rd, rd)

    def fast_s(self, tau):
        if not tau < np.finfo(np.float32).max:
            return np.float32(np.inf)
        t = div(tau, self.omg_rd, ru)
        v = max(t if self.l1 else sqrt_ru(t), np.float32(1e-30 if self.l1 else 1e-18))
        return mul(v, np.float32(float(MARGIN)), rn)

    def lb2_term(self, sm, chi0, fused):
        p = mul(sm, self.opc_ru, rn)
        if not (np.isfinite(p) and np.isfinite(chi0)):
            return np.float32(np.inf)
        if fused:
            return rn(fr(p) * MARGIN + fr(chi0))
        return add(mul(p, np.float32(float(MARGIN)), rn), chi0, rn)

    def fast_reject(self, sm, lb2, hpsi):
        s = add(sm, hpsi, rn)
        L = mul(min(s, lb2), np.float32(float(MARGIN)), rn)
        D = L if self.l1 else mul(L, L, rn)
        return mul(mul(D, self.opg_ru, rn), np.float32(float(MARGIN)), rn)


def logu(rng, lo, hi):
    return np.float32(10.0 ** rng.uniform(lo, hi))


@pytest.mark.parametrize("l1", [False, True])
@pytest.mark.parametrize("dp", [16, 128, 1024])
def test_fast_rejection_prunes_only_what_the_full_bound_prunes(dp, l1):
    rng = random.Random(dp * 2 + l1)
    plan = Plan(dp, l1)
    checked = fast = 0
    specials = [np.float32(0), np.float32(1e-40), np.float32(1e-36), np.finfo(np.float32).max]
    for i in range(700):
        tau = specials[i % 4] if i < 12 else logu(rng, -25, 25)
        chi0 = plan.query_term(logu(rng, -25, 25) if i % 5 else np.float32(0))
        hpsi = plan.psi_bound(logu(rng, -25, 25) if i % 7 else np.float32(0))
        for fused in (False, True):
            sm = plan.fast_s(tau)
            limit = plan.fast_reject(sm, plan.lb2_term(sm, chi0, fused), hpsi)
            cands = [logu(rng, -30, 30) for _ in range(3)]
            if np.isfinite(limit):
                v = np.float32(limit)
                for _ in range(3):  # just past the limit, where a violation would show
                    v = _up(v)
                    if np.isfinite(v):
                        cands.append(v)
            for dqr in cands:
                if not dqr > limit:
                    continue
                fast += 1
                thr = plan.prune_threshold(dqr, chi0, hpsi)
                assert thr > tau, (dp, l1, fused, float(tau), float(chi0), float(hpsi), float(dqr), float(thr))
            checked += 1
    assert checked == 1400 and fast > 500  # the test ran and the fast path prunes often
