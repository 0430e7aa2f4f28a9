"""Binomial checkpointing of a time loop for its adjoint (host logic).

Reversing ``t`` steps with ``c`` stored states (the initial state included)
needs at least

    T(t, c) = r t - beta(c + 1, r - 1),   beta(c, r) = (c + r)! / (c! r!),

forward re-steps, r being the least integer with beta(c, r) >= t
(Griewank's binomial bound).  This equals the recursion
T(t, c) = min_l [l + T(t - l, c - 1) + T(l, c)], T(1, c) = 0,
T(t, 1) = t (t - 1) / 2, of "advance l steps, store, reverse the right
part with one state fewer, then the left part".  ``schedule`` emits that
recursion with the split l chosen by minimising the closed form, so it
meets the bound exactly.  The adjoint of step i is taken with the state of
step i current (no forward re-step inside it), which is what T counts.

Actions:
  ("restore", i)     make stored state i current
  ("advance", i, j)  step the current state from i to j
  ("store", i)       keep the current state (at i)
  ("free", i)        drop stored state i
  ("adjoint", i)     reverse step i (state i is current)
"""

from __future__ import annotations

from math import comb

__all__ = ["binomial_cost", "schedule", "simulate"]


def _beta(c, r):
    return comb(c + r, c)


def _reps(t, c):
    r = 0
    while _beta(c, r) < t:
        r += 1
    return r


def binomial_cost(t, c):
    """Least number of forward re-steps reversing t steps with c stored states."""
    if t < 1 or c < 1:
        raise ValueError("need t >= 1 steps and c >= 1 stored states")
    if t == 1:
        return 0
    if c == 1:
        return t * (t - 1) // 2
    r = _reps(t, c)
    return r * t - _beta(c + 1, r - 1)


def _split(t, c):
    best, arg = None, 1
    for l in range(1, t):
        v = l + binomial_cost(t - l, c - 1) + binomial_cost(l, c)
        if best is None or v < best:
            best, arg = v, l
    return arg


def schedule(nsteps, snaps):
    """Action list reversing steps nsteps-1 .. 0 with at most ``snaps`` stored
    states; state 0 is stored first."""
    if nsteps < 1 or snaps < 1:
        raise ValueError("need nsteps >= 1 and snaps >= 1")
    out = [("store", 0)]
    if snaps >= nsteps:
        # every state fits: one forward sweep storing each, then the adjoints
        # in reverse order, each state dropped once reversed (t - 1 steps,
        # the bound at c >= t)
        for i in range(nsteps - 1):
            out += [("advance", i, i + 1), ("store", i + 1)]
        for i in range(nsteps - 1, -1, -1):
            out += [("restore", i), ("adjoint", i)]
            if i:
                out.append(("free", i))
        return out
    cache = {}

    def split(t, c):
        key = (t, c)
        if key not in cache:
            cache[key] = _split(t, c)
        return cache[key]

    def rev(a, b, c):
        if b - a == 1:
            out.append(("restore", a))
            out.append(("adjoint", a))
            return
        if c == 1:
            for i in range(b - 1, a - 1, -1):
                out.append(("restore", a))
                if i > a:
                    out.append(("advance", a, i))
                out.append(("adjoint", i))
            return
        m = a + split(b - a, c)
        out.append(("restore", a))
        out.append(("advance", a, m))
        out.append(("store", m))
        rev(m, b, c - 1)
        out.append(("free", m))
        rev(a, m, c)

    rev(0, nsteps, min(snaps, nsteps))
    return out


def simulate(actions):
    """Check an action list: returns (forward re-steps, peak stored states,
    order of reversed steps); raises ValueError on an inconsistent list."""
    stored, cur, steps, peak, order = set(), 0, 0, 0, []
    for act in actions:
        kind = act[0]
        if kind == "store":
            if cur is None or cur != act[1]:
                raise ValueError(f"store of state {act[1]} while {cur} is current")
            stored.add(act[1])
            peak = max(peak, len(stored))
        elif kind == "restore":
            if act[1] not in stored:
                raise ValueError(f"restore of state {act[1]} that is not stored")
            cur = act[1]
        elif kind == "advance":
            if cur != act[1] or act[2] <= act[1]:
                raise ValueError(f"advance {act[1]}->{act[2]} while {cur} is current")
            steps += act[2] - act[1]
            cur = act[2]
        elif kind == "free":
            stored.discard(act[1])
        elif kind == "adjoint":
            if cur != act[1]:
                raise ValueError(f"adjoint of step {act[1]} while {cur} is current")
            order.append(act[1])
            cur = None
        else:
            raise ValueError(f"unknown action {act!r}")
    return steps, peak, order
