"""When to save or do things during ``hysteresis`` / ``relax``
(interface/nsim/when.py).

A schedule is built from ``at(identifier, value)`` and
``every(identifier, delta, first=0, last=None)``, combined with ``|`` and
``&``; ``never`` never fires.  Identifiers are the clock's counters: ``step``,
``stage_step``, ``time``, ``stage_time`` (SI seconds or simulation units),
``real_time`` (seconds), ``stage`` and the flags ``convergence`` and
``stage_end``.

Each schedule answers two questions about a clock (a mapping identifier ->
value):

* ``match_time(clock)``: does it fire now?
* ``next_time(identifier, clock)``: the next value of that counter at which it
  fires, ``False`` if it never will, ``True`` if it does not depend on that
  counter (when.py:19-147).

Times given as SI objects are converted to simulation units once, so the
clock carries plain floats.
"""
from __future__ import annotations

from .si import SI, simulation_units

_TIME_IDS = ("time", "stage_time")


def _is_integer(x):
    # when.py:6-9: x is an integer up to the rounding of a ratio of floats
    return 1.0 + (x - round(x)) * 0.5 == 1.0


def _su(identifier, v):
    if v is None or not isinstance(v, SI):
        return v
    if identifier in _TIME_IDS:
        return simulation_units.of(v, compatible_with=SI("s"))
    return float(v)


class When(object):
    """Base of the schedules; ``a | b`` fires when either does, ``a & b`` when
    both do."""

    def match_time(self, clock):
        raise NotImplementedError

    def _next(self, identifier, clock):
        raise NotImplementedError

    def next_time(self, identifier, clock, tols=None):
        """when.py:161-179: with a tolerance for the identifier, a next time
        within it of the current value is skipped (rounding of sums of
        floating-point times)."""
        nt = self._next(identifier, clock)
        if tols and identifier in tols and not isinstance(nt, bool):
            tol, now = tols[identifier], clock[identifier]
            if tol > 0.0 and abs(nt - now) < tol:
                probe = dict(clock)
                probe[identifier] = nt + tol
                return self._next(identifier, probe)
        return nt

    def __or__(self, other):
        return _Or(self, other)

    def __and__(self, other):
        return _And(self, other)


class _At(When):
    def __init__(self, identifier, value):
        self.identifier, self.value = identifier, _su(identifier, value)

    def match_time(self, clock):
        return clock[self.identifier] == self.value

    def _next(self, identifier, clock):
        if identifier != self.identifier:
            return True
        t = clock[identifier]
        if isinstance(t, bool):
            return t == self.value
        return self.value if t < self.value else False

    def __repr__(self):
        return "at(%s, %s)" % (self.identifier, self.value)


class _Every(When):
    def __init__(self, identifier, delta, first, last):
        self.identifier = identifier
        self.delta, self.first, self.last = (_su(identifier, delta), _su(identifier, first), _su(identifier, last))

    def match_time(self, clock):
        t = clock[self.identifier]
        if self.first is not None and t < self.first:
            return False
        if self.last is not None and t > self.last:
            return False
        if self.delta is None:
            return True
        return _is_integer(float(t - self.first) / self.delta)

    def _next(self, identifier, clock):
        if identifier != self.identifier:
            return self.match_time(clock)
        t = clock[identifier]
        if self.last is not None and t >= self.last:
            return False
        if self.first is not None and t < self.first and self.delta is not None:
            return self.first
        if self.delta is None:
            return True
        pos = float(t - self.first) / self.delta
        k = int(round(pos)) + 1 if _is_integer(pos) else int(pos) + 1
        nxt = self.delta * k + self.first
        if self.last is not None and nxt > self.last:
            return False
        return nxt

    def __repr__(self):
        return "every(%s, %s, first=%s, last=%s)" % (self.identifier, self.delta, self.first, self.last)


class _Or(When):
    def __init__(self, a, b):
        self.a, self.b = a, b

    def match_time(self, clock):
        return self.a.match_time(clock) or self.b.match_time(clock)

    def _next(self, identifier, clock):
        n1, n2 = self.a._next(identifier, clock), self.b._next(identifier, clock)
        b1, b2 = isinstance(n1, bool), isinstance(n2, bool)
        if b1 and b2:
            return n1 or n2
        if b1:
            return n2
        if b2:
            return n1
        return min(n1, n2)

    def __repr__(self):
        return "%r | %r" % (self.a, self.b)


class _And(When):
    """Both schedules fire: the first value of the counter at which the one
    that fires later also makes the other match (when.py:98-128).  Like the
    reference, meant for independent counters."""

    def __init__(self, a, b):
        self.a, self.b = a, b

    def match_time(self, clock):
        return self.a.match_time(clock) and self.b.match_time(clock)

    def _next(self, identifier, clock, max_rounds=100000):
        probe = dict(clock)
        for _ in range(max_rounds):
            n1, n2 = self.a._next(identifier, probe), self.b._next(identifier, probe)
            if n1 is False or n2 is False:
                return False
            if n1 is True:
                return n2
            if n2 is True:
                return n1
            (hi, lo_sched) = (n1, self.b) if n1 > n2 else (n2, self.a)
            probe[identifier] = hi
            if lo_sched.match_time(probe):
                return hi
        return False

    def __repr__(self):
        return "%r & %r" % (self.a, self.b)


class _Never(When):
    def match_time(self, clock):
        return False

    def _next(self, identifier, clock):
        return False

    def __repr__(self):
        return "never"


def at(identifier, value=True):
    """Fire when the counter equals value: at('convergence'),
    at('step', 10), at('stage_time', SI(1e-11, 's'))."""
    return _At(identifier, value)


def every(arg1, arg2=None, first=0, last=None):
    """Fire periodically: every('step', 10), every('step', 5, first=10,
    last=100), every('time', SI(1e-12, 's')) (also every(10, 'step'))."""
    identifier, delta = (arg1, arg2) if isinstance(arg1, str) else (arg2, arg1)
    if not isinstance(identifier, str):
        raise ValueError("every: give an identifier, e.g. every('step', 10)")
    if last is not None and _su(identifier, last) <= _su(identifier, first):
        raise ValueError("every: last must be greater than first (first=%s, last=%s)" % (first, last))
    if delta is not None and _su(identifier, delta) <= 0:
        raise ValueError("every: the delta must be positive")
    return _Every(identifier, delta, first, last)


never = _Never()
