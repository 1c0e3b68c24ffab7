"""MagMaterial (interface/nmag/main.py:257-495); the anisotropies it takes
are in ``anisotropy.py`` (interface/nmag/anisotropy.py).

Material constants are converted to simulation units exactly as the
reference does (main.py:419-465) and then turned into the coefficients its
generated code computes with:

* operator-string constants (Ms, the exchange prefactor) pass through Python
  2's ``str(float)`` -- 12 significant digits (preprocess.py substitutor);
* local-equation coefficients (the LLG C1 ... C5 and the energy factors) are
  printed with ``%g`` -- 6 significant digits -- into generated C
  (nsim.ml:846);
* the energy factor mu0 is printed with ``%f`` (nmag_lam.py:454-459);
* anisotropy polynomials (every anisotropy but the second-order uniaxial one,
  which the engine evaluates in closed form) are printed with ``%f``
  (nsim_anisotropy.ml:189-206).

``quirks="nmag"`` (the default) reproduces these roundings; ``quirks=None``
keeps the exact double values.
"""
from __future__ import annotations

import math

from . import si as _si
from .anisotropy import PredefinedAnisotropy, cubic_anisotropy, polynomial_tables, uniaxial_anisotropy
from .si import SI, g6, py2str, f6, simulation_units

__all__ = ["MagMaterial", "PredefinedAnisotropy", "uniaxial_anisotropy", "cubic_anisotropy"]


class MagMaterial(object):
    """A magnetic material (main.py:347-473)."""

    def __init__(self, name, Ms=SI(0.86e6, "A/m"), llg_damping=0.5, llg_gamma_G=SI(2.210173e5, "m/A s"),
                 llg_normalisationfactor=SI(0.1e12, "1/s"), llg_xi=0.0, llg_polarisation=0.0, do_precession=True,
                 exchange_coupling=SI(1.3e-11, "J/m"), anisotropy=None, anisotropy_order=None,
                 properties=("magnetic", "material"), scale_volume_charges=1.0):
        self.name = name
        self.Ms = Ms
        self.llg_damping = llg_damping
        self.llg_gamma_G = llg_gamma_G
        self.llg_normalisationfactor = llg_normalisationfactor
        self.llg_xi = llg_xi
        self.llg_polarisation = llg_polarisation
        self.do_precession = do_precession
        self.exchange_coupling = exchange_coupling
        self.properties = list(properties)
        self.scale_volume_charges = float(scale_volume_charges)
        if self.scale_volume_charges != 1.0:
            raise NotImplementedError("scale_volume_charges != 1 (a developer debugging knob) is not supported")
        # main.py:408-421: a predefined anisotropy brings its order; a custom
        # energy function E(m) (J/m^3) needs anisotropy_order
        if isinstance(anisotropy, PredefinedAnisotropy):
            if anisotropy_order:
                raise ValueError("Cannot specify custom anisotropy_order when using a predefined anisotropy.")
            self.anisotropy = anisotropy
            self.anisotropy_order = anisotropy.order
        elif anisotropy is not None:
            if not anisotropy_order:
                raise ValueError("You need to specify the anisotropy_order when using a custom anisotropy function.")
            self.anisotropy = PredefinedAnisotropy(anisotropy, int(anisotropy_order))
            self.anisotropy_order = int(anisotropy_order)
        else:
            self.anisotropy = None
            self.anisotropy_order = None
        self._compute_su()

    def _compute_su(self):
        su = simulation_units
        self.su_Ms = su.of(self.Ms, compatible_with=SI("A/m"))
        self.su_llg_gamma_G = su.of(self.llg_gamma_G, compatible_with=SI("m/A s"))
        self.su_llg_damping = float(self.llg_damping)
        self.su_llg_normalisationfactor = su.of(self.llg_normalisationfactor, compatible_with=SI("1/s"))
        self.su_exchange_coupling = su.of(self.exchange_coupling, compatible_with=SI("J/m"))
        if self.su_exchange_coupling < 0.0:
            raise ValueError("The exchange coupling constant must be positive.")
        gilbert_to_ll = 1.0 / (1.0 + self.su_llg_damping ** 2)
        self.su_llg_coeff1 = -self.su_llg_gamma_G * gilbert_to_ll
        self.su_llg_coeff2 = self.su_llg_coeff1 * self.su_llg_damping
        if not self.do_precession:
            self.su_llg_coeff1 = 0.0
        # spin-transfer torque (main.py:440-451): Zhang-Li coefficients of
        # m x (m x (J.grad)m) (adiabatic) and m x (J.grad)m (non-adiabatic)
        su_xi = su.of(self.llg_xi, compatible_with=SI(""))
        su_pol = su.of(self.llg_polarisation, compatible_with=SI(""))
        su_f = -gilbert_to_ll * (su_pol * su.of(_si.bohr_magneton)
                                 / (su.of(_si.positron_charge) * self.su_Ms * (1.0 + su_xi * su_xi)))
        self.su_llg_stt_prefactor = 0.0 if su_f == 0.0 else 1.0
        self.su_llg_stt_nadiab = su_f * (su_xi - self.su_llg_damping)
        self.su_llg_stt_adiab = su_f * (1.0 + self.su_llg_damping * su_xi)
        self.su_mu0 = su.of(_si.mu0)
        self.su_exch_prefactor = 2.0 * self.su_exchange_coupling / (self.su_mu0 * self.su_Ms)
        self.su_K1 = 0.0
        self.axis = (0.0, 0.0, 1.0)
        self._poly = {}
        if self.anisotropy is not None and self.anisotropy.closed_form_uniaxial():
            K1 = self.anisotropy.K1
            self.su_K1 = su.of(K1, compatible_with=SI("J/m^3")) if isinstance(K1, SI) else float(K1)
            self.axis = tuple(self.anisotropy.axis1)

    def anisotropy_polynomial(self, quirks="nmag"):
        """Tables of nmg_set_anisotropy_poly for every anisotropy other than
        the closed-form second-order uniaxial one, else None
        (nmag_lam.py:485-502: energy fitted on the unit sphere, field =
        -(1/mu0 Ms) times its tangential gradient)."""
        if self.anisotropy is None or self.anisotropy.closed_form_uniaxial():
            return None
        if quirks not in self._poly:
            self._poly[quirks] = polynomial_tables(self.anisotropy.function, self.anisotropy_order,
                                                   1.0 / (self.su_mu0 * self.su_Ms), quirks)
        return self._poly[quirks]

    def set_damping(self, llg_damping):
        self.llg_damping = llg_damping
        self._compute_su()

    def coefficients(self, quirks="nmag"):
        """The constants the engine computes with (see module docstring)."""
        q = quirks == "nmag"
        Ms = py2str(self.su_Ms) if q else self.su_Ms
        mu0f = f6(self.su_mu0) if q else self.su_mu0
        c = {
            "Ms": Ms,
            "exch_coeff": py2str(self.su_exch_prefactor) if q else self.su_exch_prefactor,
            "C1": g6(py2str(self.su_llg_coeff1)) if q else self.su_llg_coeff1,
            "C2": g6(py2str(self.su_llg_coeff2)) if q else self.su_llg_coeff2,
            "C3": g6(py2str(self.su_llg_normalisationfactor)) if q else self.su_llg_normalisationfactor,
            "K1": self.su_K1,
            "axis": tuple(self.axis),
            "anis_coeff": 2.0 * self.su_K1 / (self.su_mu0 * self.su_Ms),
            "E_coeff_half": g6(-0.5 * Ms * mu0f) if q else -0.5 * Ms * mu0f,
            "E_coeff_ext": g6(-1.0 * Ms * mu0f) if q else -1.0 * Ms * mu0f,
            "anis_poly": self.anisotropy_polynomial(quirks),
            # LLG_C4 / LLG_C5 (nmag_lam.py:260-261), 0 without a polarisation
            "C4": g6(py2str(self.su_llg_stt_adiab)) if q else self.su_llg_stt_adiab,
            "C5": g6(py2str(self.su_llg_stt_nadiab)) if q else self.su_llg_stt_nadiab,
        }
        return c

    def __repr__(self):
        return "MagMaterial(%r, Ms=%r, llg_damping=%r)" % (self.name, self.Ms, self.llg_damping)
