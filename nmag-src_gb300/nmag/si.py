"""SI quantities and nmag's simulation units.

Mirrors the parts of ``nsim.si_units`` (interface/nsim/si_units/lib.py) and
``nsim.su_units`` (interface/nsim/su_units.py) that the LLG path needs: an
``SI`` value with dimensions, unit-string parsing ("A/m", "m/A s", "J/m^3",
"s^(-1)"), the physical constants used by ``MagMaterial``, and
``SimulationUnits.of`` which converts an SI value into the simulation's
internal units (default: A=1e-3, kg=1e-27, m=1e-9, s=1e-12, main.py:188-196).
"""
from __future__ import annotations

import math
import re

_BASE = ("m", "s", "A", "kg", "K", "mol", "cd")

# derived units expressed in base dimensions (exponent tuples over _BASE) and factor
_DERIVED = {
    "m": (1.0, {"m": 1}), "s": (1.0, {"s": 1}), "A": (1.0, {"A": 1}), "kg": (1.0, {"kg": 1}),
    "K": (1.0, {"K": 1}), "mol": (1.0, {"mol": 1}), "cd": (1.0, {"cd": 1}),
    "J": (1.0, {"kg": 1, "m": 2, "s": -2}),
    "N": (1.0, {"kg": 1, "m": 1, "s": -2}),
    "W": (1.0, {"kg": 1, "m": 2, "s": -3}),
    "T": (1.0, {"kg": 1, "s": -2, "A": -1}),
    "H": (1.0, {"kg": 1, "m": 2, "s": -2, "A": -2}),
    "V": (1.0, {"kg": 1, "m": 2, "s": -3, "A": -1}),
    "C": (1.0, {"A": 1, "s": 1}),
    "Ohm": (1.0, {"kg": 1, "m": 2, "s": -3, "A": -2}),
}
_PREFIX = {"": 1.0, "m": 1e-3, "u": 1e-6, "n": 1e-9, "p": 1e-12, "f": 1e-15, "k": 1e3, "M": 1e6, "G": 1e9}


def _parse_units(spec: str):
    """Parse a unit string such as "m/A s" or "J/m^3" or "s^(-1)".

    Everything after a "/" is in the denominator (nsim's convention:
    "m/A s" == m A^-1 s^-1)."""
    spec = spec.strip()
    factor, dims = 1.0, {}
    if spec in ("", "1"):
        return factor, dims
    num, _, den = spec.partition("/")
    for part, sign in ((num, 1), (den, -1)):
        for tok in part.replace("*", " ").split():
            if tok == "1":
                continue
            mt = re.fullmatch(r"([A-Za-z]+)(?:\^\(?(-?\d+)\)?)?", tok)
            if not mt:
                raise ValueError("bad unit token %r in %r" % (tok, spec))
            name, p = mt.group(1), int(mt.group(2) or 1)
            if name in _DERIVED:
                f, d = _DERIVED[name]
            elif name[0] in _PREFIX and name[1:] in _DERIVED and len(name) > 1:
                f, d = _DERIVED[name[1:]]
                f = f * _PREFIX[name[0]]
            else:
                raise ValueError("unknown unit %r" % name)
            factor *= f ** (sign * p)
            for k, v in d.items():
                dims[k] = dims.get(k, 0) + sign * p * v
    return factor, {k: v for k, v in dims.items() if v}


class SI(object):
    """A value with SI dimensions: ``SI(0.86e6, "A/m")``."""

    __slots__ = ("value", "dims")

    def __init__(self, value=1.0, units=""):
        if isinstance(value, str) and units == "":
            value, units = 1.0, value   # SI("A/m") is the unit itself
        if isinstance(units, dict):
            f, d = 1.0, dict(units)
        elif isinstance(units, (list, tuple)):
            f, d = 1.0, {}
            for k, v in zip(units[0::2], units[1::2]):
                d[k] = d.get(k, 0) + v
        else:
            f, d = _parse_units(units)
        self.value = float(value) * f
        self.dims = {k: v for k, v in d.items() if v}

    def _new(self, value, dims):
        r = SI.__new__(SI)
        r.value, r.dims = value, {k: v for k, v in dims.items() if v}
        return r

    def is_compatible_with(self, other):
        od = other.dims if isinstance(other, SI) else {}
        return self.dims == od

    def __mul__(self, o):
        if isinstance(o, SI):
            d = dict(self.dims)
            for k, v in o.dims.items():
                d[k] = d.get(k, 0) + v
            return self._new(self.value * o.value, d)
        return self._new(self.value * float(o), self.dims)

    __rmul__ = __mul__

    def __truediv__(self, o):
        if isinstance(o, SI):
            d = dict(self.dims)
            for k, v in o.dims.items():
                d[k] = d.get(k, 0) - v
            return self._new(self.value / o.value, d)
        return self._new(self.value / float(o), self.dims)

    def __rtruediv__(self, o):
        return self._new(float(o) / self.value, {k: -v for k, v in self.dims.items()})

    def __add__(self, o):
        # a zero of any dimension is neutral (lib.py:380-399 accepts it too),
        # so that e.g. -K1 a^2 - K2 a^4 with K2 = 0 stays an energy density
        if not isinstance(o, SI):
            if float(o) == 0.0:
                return self
            if not self.dims:
                return self._new(self.value + float(o), self.dims)
            raise ValueError("incompatible SI addition")
        if o.dims != self.dims:
            if o.value == 0.0:
                return self
            if self.value == 0.0:
                return o
            raise ValueError("incompatible SI addition")
        return self._new(self.value + o.value, self.dims)

    __radd__ = __add__

    def __sub__(self, o):
        return self + (-1.0) * o

    def __rsub__(self, o):
        return (-self) + o

    def __neg__(self):
        return self._new(-self.value, self.dims)

    def __pow__(self, p):
        return self._new(self.value ** p, {k: v * p for k, v in self.dims.items()})

    def __float__(self):
        if self.dims:
            raise ValueError("SI quantity with dimensions %s is not a float" % self.dims)
        return self.value

    def __repr__(self):
        u = " ".join("%s^%d" % (k, v) if v != 1 else k for k, v in sorted(self.dims.items()))
        return "SI(%r, %r)" % (self.value, u)

    # the rest of the reference's Physical interface (si_units/lib.py:330-470)
    def in_units_of(self, unit):
        """This quantity as a multiple of ``unit`` (compatible units)."""
        u = unit if isinstance(unit, SI) else SI(float(unit))
        if u.dims != self.dims:
            raise ValueError("%r is not compatible with %r" % (self, u))
        return self.value / u.value

    def get_units(self):
        """The units of this quantity (value 1)."""
        return self._new(1.0, self.dims)

    def copy(self):
        return self._new(self.value, self.dims)

    def _cmp_value(self, o):
        # zero compares with any dimension (lib.py:364-374)
        if not isinstance(o, SI):
            o = SI(float(o))
        if o.dims != self.dims and self.value != 0.0 and o.value != 0.0:
            raise ValueError("Expected quantities of matching dimensions: %r and %r" % (self, o))
        return o.value

    def __lt__(self, o):
        return self.value < self._cmp_value(o)

    def __le__(self, o):
        return self.value <= self._cmp_value(o)

    def __gt__(self, o):
        return self.value > self._cmp_value(o)

    def __ge__(self, o):
        return self.value >= self._cmp_value(o)

    def __eq__(self, o):
        if not isinstance(o, SI):
            return False
        return self.dims == o.dims and self.value == o.value

    def __ne__(self, o):
        return not self.__eq__(o)

    __hash__ = None

    def __abs__(self):
        return self._new(abs(self.value), self.dims)

    def __pos__(self):
        return self.copy()

    def __str__(self):
        """'<SI: 1e+06  A / m >' (lib.py:376-395)."""
        def part(sign):
            out = ""
            for u in ("m", "kg", "s", "A", "K", "mol", "cd"):
                p = self.dims.get(u, 0)
                if p and (p > 0) == (sign > 0):
                    out += " %s" % u if abs(p) == 1 else " %s^%d" % (u, abs(p))
            return out
        powers = part(+1)
        neg = part(-1)
        if neg:
            powers = "%s /%s" % (powers, neg)
        return "<SI: %g %s >" % (self.value, powers)

    def dens_str(self, angles=True):
        """si_units/lib.py:304-340: '<A/m>', '<kg/ms^2>', '<1e-09m>': positive
        then negative powers in the order m kg s A K mol cd, no separators."""
        def part(sign):
            out = ""
            for u in ("m", "kg", "s", "A", "K", "mol", "cd"):
                p = self.dims.get(u, 0)
                if p and (p > 0) == (sign > 0):
                    out += u if abs(p) == 1 else "%s^%d" % (u, abs(p))
            return out
        powers = part(+1)
        neg = part(-1)
        if neg:
            powers = "%s/%s" % (powers, neg)
        body = (powers or "1") if self.value == 1.0 else "%g%s" % (self.value, powers)
        return "<%s>" % body if angles else body


# units and physical constants (interface/nsim/si_units/si.py)
kilogram = SI(1.0, "kg")
meter = metre = SI(1.0, "m")
Ampere = SI(1.0, "A")
Kelvin = SI(1.0, "K")
second = SI(1.0, "s")
candela = SI(1.0, "cd")
mol = SI(1.0, "mol")
Newton = kilogram * meter / second ** 2
Joule = SI(1.0, "J")
Tesla = kilogram / Ampere / second ** 2
Gauss = 1e-4 * Tesla
mu0 = SI(4.0e-7 * math.pi, "N/A^2")
Oersted = Oe = Gauss / mu0
gamma0 = SI(-2.2137286285040001e5, "m/A s")
positron_charge = SI(1.6021765314e-19, "C")
electron_charge = -positron_charge
plank_constant = 6.6260689633e-34 * Joule * second
reduced_plank_constant = plank_constant / (2 * math.pi)
bohr_magneton = SI(9.2740094980e-24, "J/T")
boltzmann_constant = SI(1.3806504e-23, "J/K")
degrees_per_ns = SI(math.pi / 180.0 / 1e-9, "1/s")


class SimulationUnits(object):
    """Simulation units: ``of(x)`` divides by the product of base-unit scales."""

    def __init__(self, scales):
        self.scales = dict(scales)

    def of(self, x, compatible_with=None):
        if not isinstance(x, SI):
            x = SI(float(x))
        if compatible_with is not None and isinstance(compatible_with, SI):
            if x.dims != compatible_with.dims:
                raise ValueError("%r is not compatible with %r" % (x, compatible_with))
        f = 1.0
        for k, v in x.dims.items():
            f *= self.scales.get(k, 1.0) ** v
        return x.value / f

    def conversion_factor_of(self, unit):
        return 1.0 / self.of(unit)


simulation_units = SimulationUnits({"A": 1e-3, "kg": 1e-27, "m": 1e-9, "s": 1e-12, "cd": 1.0, "K": 1.0, "mol": 1.0})


def str_of_SI_vector(v):
    """'[1e+06 0 0]<A/m>' (si_units/lib.py str_of_SI_vector): the values with
    %g and the common unit once; plain zeros may stand among SI values."""
    if v is None:
        return "None"
    dims = None
    vals = []
    for x in v:
        if isinstance(x, SI):
            if dims is None or (not any(dims.values()) and x.dims):
                dims = x.dims
            vals.append(x.value)
        else:
            vals.append(float(x))
    unit = SI(1.0, dict(dims or {})).dens_str()
    return "[%s]%s" % (" ".join("%g" % x for x in vals), unit)


def g6(x: float) -> float:
    """Round like C's printf("%g") (6 significant digits).

    nsim prints local-equation coefficients with %g into generated C code
    (nsim.ml:846); the value it computes with is this rounded one."""
    return float("%g" % float(x))


def py2str(x: float) -> float:
    """Round like Python 2's str(float) (12 significant digits), which nmag's
    template preprocessor uses to put material constants into operator strings
    (interface/nsim/preprocess.py substitutor)."""
    return float("%.12g" % float(x))


def f6(x: float) -> float:
    """Round like printf("%f") (6 decimals): anisotropy and energy-factor
    coefficients (nsim_anisotropy.ml:211, nmag_lam.py:454-459)."""
    return float("%f" % float(x))
