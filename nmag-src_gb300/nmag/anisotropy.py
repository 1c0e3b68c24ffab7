"""Anisotropies (interface/nmag/anisotropy.py) and the polynomial form the
engine evaluates (src/nsim_anisotropy.ml).

The reference turns every anisotropy energy density E(m) into polynomials in
the magnetisation components:

1. E is represented on the unit sphere by a homogeneous polynomial of degree
   ``order``, sum_p c_p mx^a my^b mz^c with a + b + c = order
   (nsim_anisotropy.ml:8-22,131-145: ``taylor_coefficients_of_spherical_
   function``; coefficients below 1e-10 dropped);
2. the field is minus the tangential gradient, H = -(1/mu0 Ms) (grad E -
   (m . grad E) m), expanded into monomials (:147-206) -- degree order - 1
   and order + 1 terms;
3. both are printed into generated C with ``%f`` (:189-206), so every
   coefficient the engine computes with is rounded to 6 decimals.

The reference finds the coefficients by interpolating E at as many random
points on the sphere as there are monomials (:51-129).  Here a least-squares
fit over a fixed, well-spread point set is used: for an energy that is a
polynomial of that degree on the sphere (every predefined anisotropy) both
give the unique homogeneous polynomial, up to rounding; for other functions
the reference's result depends on its random points and this fit is the
best approximation in the mean.

Exponents reach the engine packed as a | b << 4 | c << 8
(``nmg_set_anisotropy_poly``).
"""
from __future__ import annotations

import itertools
import math

import numpy as np

from .si import SI, f6, simulation_units

MAX_ORDER = 12   # field terms reach degree order + 1 <= 13 (the engine's power tables)


class PredefinedAnisotropy(object):
    """An anisotropy energy function with its polynomial order
    (anisotropy.py:25-90).  Sums, differences and negations of objects that
    carry a function are anisotropies again (order the larger one)."""

    def __init__(self, function=None, order=None, anis_type="functional", axis1=None, axis2=None, axis3=None,
                 K1=None, K2=None, K3=None, stringifier=None):
        if function is None and order is None:
            raise ValueError("Please specify a sampling order.")
        self.anis_type = anis_type
        self.function = function
        self.order = order
        self.K1, self.K2, self.K3 = K1, K2, K3
        self.axis1, self.axis2, self.axis3 = axis1, axis2, axis3
        self._str_extra = stringifier

    def has_function(self):
        return self.function is not None

    def _other(self, y):
        if not isinstance(y, PredefinedAnisotropy) or not y.has_function():
            raise ValueError("%s <-- not an anisotropy with an energy function" % (y,))
        return y

    def __neg__(self):
        return PredefinedAnisotropy(lambda m: -self.function(m), self.order)

    def __pos__(self):
        return self

    def __add__(self, y):
        y = self._other(y)
        return PredefinedAnisotropy(lambda m: self.function(m) + y.function(m), max(self.order, y.order))

    def __sub__(self, y):
        y = self._other(y)
        return PredefinedAnisotropy(lambda m: self.function(m) - y.function(m), max(self.order, y.order))

    def closed_form_uniaxial(self):
        """True for a second-order uniaxial anisotropy, which the engine
        evaluates in closed form (nmg_material K1 / axis)."""
        return self.anis_type == "uniaxial" and self.order == 2

    def __repr__(self):
        s = self._str_extra(self) if self._str_extra else "?"
        return 'PredefinedAnisotropy(anis_type="%s", %s)' % (self.anis_type, s)


def _normalised(v):
    v = [float(x) for x in v]
    n = math.sqrt(sum(x * x for x in v))
    if n == 0.0:
        raise ValueError("zero-length anisotropy axis")
    return [x / n for x in v]


def _cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def _dot(a, m):
    return a[0] * m[0] + a[1] * m[1] + a[2] * m[2]


def uniaxial_anisotropy(axis, K1, K2=0):
    """E_anis = -K1 <axis, m>^2 - K2 <axis, m>^4 (anisotropy.py:92-137);
    order 4 when K2 is given, else 2."""
    axis = _normalised(axis)

    def f(m):
        a = _dot(axis, m)
        return -K1 * a ** 2 - K2 * a ** 4

    def stringifier(a):
        s = "axis=[%s, %s, %s], K1=%s" % tuple(list(a.axis1) + [a.K1])
        return s + (", %s" % a.K2 if a.K2 else "")

    return PredefinedAnisotropy(f, 4 if K2 else 2, "uniaxial", axis1=axis, K1=K1, K2=K2, stringifier=stringifier)


def cubic_anisotropy(axis1, axis2, K1, K2=0, K3=0):
    """E_anis = K1 (a1^2 a2^2 + a1^2 a3^2 + a2^2 a3^2) + K2 a1^2 a2^2 a3^2
    + K3 (a1^4 a2^4 + a1^4 a3^4 + a2^4 a3^4), a_k = <axis_k, m>, with axis2
    orthogonalised against axis1 and axis3 = axis1 x axis2
    (anisotropy.py:140-200); order 8 with K3, 6 with K2, else 4."""
    axis3 = _cross(axis1, axis2)
    axis2 = _cross(axis3, axis1)
    axis1, axis2, axis3 = (_normalised(v) for v in (axis1, axis2, axis3))

    def f(m):
        a1, a2, a3 = _dot(axis1, m), _dot(axis2, m), _dot(axis3, m)
        return (K1 * ((a1 * a2) ** 2 + (a1 * a3) ** 2 + (a2 * a3) ** 2)
                + K2 * ((a1 * a2 * a3) ** 2)
                + K3 * ((a1 * a2) ** 4 + (a1 * a3) ** 4 + (a2 * a3) ** 4))

    def stringifier(a):
        s = "axis1=[%s, %s, %s], axis2=[%s, %s, %s], K1=%s" % tuple(list(a.axis1) + list(a.axis2) + [a.K1])
        s += ", %s" % a.K2 if a.K2 else ""
        return s + (", %s" % a.K3 if a.K3 else "")

    order = 8 if K3 else (6 if K2 else 4)
    return PredefinedAnisotropy(f, order, "cubic", axis1=axis1, axis2=axis2, axis3=axis3, K1=K1, K2=K2, K3=K3,
                                stringifier=stringifier)


def su_energy_function(function):
    """E(m) in simulation units (main.py:466-470): SI results are converted
    from J/m^3, plain numbers are taken as simulation units."""
    def f(m):
        v = function(m)
        if isinstance(v, SI):
            return simulation_units.of(v, compatible_with=SI("J/m^3")) if v.value != 0.0 else 0.0
        return float(v)
    return f


def monomials(order):
    """Exponent triples (a, b, c) with a + b + c = order."""
    return [(a, b, order - a - b) for a in range(order, -1, -1) for b in range(order - a, -1, -1)]


def _points(n):
    # fixed, well-spread points on the unit sphere (a Fibonacci lattice)
    k = np.arange(n) + 0.5
    z = 1.0 - 2.0 * k / n
    r = np.sqrt(1.0 - z * z)
    phi = k * math.pi * (3.0 - math.sqrt(5.0))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def spherical_polynomial(f_su, order):
    """Coefficients of the homogeneous polynomial of degree ``order`` equal to
    f_su on the unit sphere: [(c, (a, b, c_exp)), ...] with |c| > 1e-10
    (nsim_anisotropy.ml:131-145)."""
    if not (isinstance(order, int) and 1 <= order <= MAX_ORDER):
        raise ValueError("anisotropy_order must be an integer in 1..%d" % MAX_ORDER)
    terms = monomials(order)
    pts = _points(max(8 * len(terms), 200))
    A = np.stack([pts[:, 0] ** a * pts[:, 1] ** b * pts[:, 2] ** c for (a, b, c) in terms], axis=1)
    y = np.array([f_su(list(p)) for p in pts], dtype=np.float64)
    coef = np.linalg.lstsq(A, y, rcond=None)[0]
    return [(float(c), t) for c, t in zip(coef, terms) if abs(c) > 1e-10]


def tangential_field(poly, factor):
    """-factor (grad E - (m . grad E) m) as three dictionaries monomial ->
    coefficient (nsim_anisotropy.ml:147-206, then the negation and the
    correction factor 1/(mu0 Ms) of :207-236)."""
    grad = [dict() for _ in range(3)]
    for c, p in poly:
        for d in range(3):
            if p[d]:
                q = list(p); q[d] -= 1; q = tuple(q)
                grad[d][q] = grad[d].get(q, 0.0) + c * p[d]
    sprod = {}
    for d in range(3):
        for q, c in grad[d].items():
            r = list(q); r[d] += 1; r = tuple(r)
            sprod[r] = sprod.get(r, 0.0) + c
    field = []
    for d in range(3):
        h = dict(grad[d])
        for q, c in sprod.items():
            r = list(q); r[d] += 1; r = tuple(r)
            h[r] = h.get(r, 0.0) - c
        field.append({q: -c * factor for q, c in h.items()})
    return field


def pack(p):
    return p[0] | (p[1] << 4) | (p[2] << 8)


def polynomial_tables(function, order, factor, quirks="nmag"):
    """The tables of nmg_set_anisotropy_poly for an energy function (SI or
    simulation units) of the given order: (e_pow, e_coef, h_pow, h_coef) as
    tuples, h_coef three per term.  quirks="nmag" rounds every coefficient
    like the reference's ``%f`` printing."""
    rnd = f6 if quirks == "nmag" else float
    poly = spherical_polynomial(su_energy_function(function), order)
    # terms in the order of the exponent triples, as the reference lists them
    # (nsim_anisotropy.ml:147-150)
    e = [(pack(p), rnd(c)) for c, p in sorted(poly, key=lambda t: t[1])]
    e = [(p, c) for p, c in e if c != 0.0]
    field = tangential_field(poly, factor)
    hp = sorted(set(itertools.chain.from_iterable(field)))
    rows = []
    for q in hp:
        cs = tuple(rnd(field[d].get(q, 0.0)) for d in range(3))
        if any(cs):
            rows.append((pack(q), cs))
    return (tuple(p for p, _ in e), tuple(c for _, c in e),
            tuple(p for p, _ in rows), tuple(c for _, cs in rows for c in cs))

