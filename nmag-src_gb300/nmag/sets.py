"""Lists of numbers and vectors for hysteresis loops (interface/nsim/sets.py).

``float_set`` reads a small language of numbers:

* ``[a, b, [], c]`` (or ``"..."`` for ``[]``): a, b and the arithmetic
  progression with step b - a continued up to c (c itself always ends it);
* ``[a, [n], c]``: n equal steps from a to c;
* pieces chain: the end of one is the start of the next, e.g.
  ``[0, [3], 3, 4, [], 6]`` -> 0, 1, 2, 3, 4, 5, 6.

``vector_set(norm_list, direction)`` scales a (normalised) direction by the
numbers of ``float_set(norm_list)``: the usual way to give the applied fields
of ``Simulation.hysteresis``.
"""
from __future__ import annotations

__all__ = ["float_set", "vector_set"]


def _scaled(units):
    return (lambda x: x) if units is None else (lambda x: x * units)


def _continue(out, first, second, last, scale):
    """Append first + i (second - first) for i >= 2 while short of last, then
    last (sets.py:12-35): the count is rounded when (last - first) is a whole
    number of steps up to rounding, else the progression stops before last."""
    step = second - first
    interval = last - first
    n = interval / step
    if n <= 1.0:
        raise ValueError("float_set: [..., %g, %g, [], %g, ...]: %g should lie between %g and %g"
                         % (first, second, last, second, first, last))
    whole = abs(interval / round(n) - step) / 64 + interval == interval
    count = int(round(n)) if whole else int(n) + 1
    for i in range(2, count):
        out.append(scale(first + i * step))
    out.append(scale(last))


def float_set(float_list, units=None):
    """The numbers the list describes (see the module docstring), multiplied
    by units when given -- except those of an ``[a, [n], b]`` range, which the
    reference leaves unscaled (sets.py:88-97)."""
    scale = _scaled(units)
    out = []
    prev2 = prev1 = None   # the last two numbers read
    mode, steps = None, 0
    for token in float_list:
        if mode is None:
            if token == "..." or (isinstance(token, list) and not token):
                if prev1 is None or prev2 is None:
                    raise ValueError("float_set: a continuation needs two numbers before it, "
                                     "as in [1, 2, [], 10]")
                mode = "continue"
            elif isinstance(token, list):
                if len(token) != 1 or not isinstance(token[0], int):
                    raise ValueError("float_set: ranging from a to b in n steps is written [a, [n], b] "
                                     "with n an integer")
                if token[0] < 1 or prev1 is None:
                    raise ValueError("float_set: [a, [n], b] needs a start a and n >= 1")
                mode, steps = "steps", token[0]
            else:
                prev2, prev1 = prev1, float(token)
                out.append(scale(prev1))
        elif mode == "continue":
            last = float(token)
            _continue(out, prev2, prev1, last, scale)
            prev2, prev1, mode = None, last, None
        else:   # n equal steps from prev1 to token (sets.py:88-97)
            # the reference appends these values without units (only its
            # other two branches scale), and a drop-in gives the same list
            last = float(token)
            h = (last - prev1) / steps
            start = prev1 + h
            for i in range(steps):
                out.append(start + i * h)
            prev2, prev1, mode = None, last, None
    if mode is not None:
        raise ValueError('float_set: the list cannot end with "...", [] or [n]')
    return out


def vector_set(norm_list, direction, units=None, normalize=True):
    """The vectors norm * direction for the norms of float_set(norm_list)
    (direction normalised first unless normalize is False), each component
    times units (sets.py:117-158)."""
    scale = _scaled(units)
    d = [float(x) for x in direction]
    if normalize:   # times the reciprocal of the norm, as sets.py:139-141 scales
        inv = 1.0 / sum(x * x for x in d) ** 0.5
        d = [inv * x for x in d]
    return [[scale(norm * x) for x in d] for norm in float_set(norm_list)]
