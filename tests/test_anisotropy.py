"""Anisotropies other than the closed-form uniaxial K1 term: the polynomial
form of nsim_anisotropy.ml (energy fitted on the unit sphere, field = minus
the tangential gradient over mu0 Ms, coefficients printed with %f), the
material routing, and the oracle's evaluation of it.  CPU only."""
import numpy as np
import pytest

import nmag
from nmag import SI
from nmag.anisotropy import pack, polynomial_tables, spherical_polynomial, su_energy_function


def eval_tables(tables, m):
    """E (n,) and H (n, 3) of nmg_set_anisotropy_poly tables at m (n, 3)."""
    e_pow, e_coef, h_pow, h_coef = tables
    m = np.asarray(m, dtype=np.float64).reshape(-1, 3)

    def mono(p):
        return m[:, 0] ** (p & 15) * m[:, 1] ** ((p >> 4) & 15) * m[:, 2] ** ((p >> 8) & 15)
    E = np.zeros(len(m))
    for p, c in zip(e_pow, e_coef):
        E += c * mono(p)
    H = np.zeros((len(m), 3))
    for p, c in zip(h_pow, np.reshape(h_coef, (-1, 3))):
        H += np.outer(mono(p), c)
    return E, H


def unit_vectors(n, seed):
    m = np.random.default_rng(seed).standard_normal((n, 3))
    return m / np.linalg.norm(m, axis=1)[:, None]


def fd_field(f_su, m, factor, eps=1e-6):
    """-factor (grad E - (m . grad E) m) by central differences."""
    out = np.zeros_like(m)
    for i, x in enumerate(m):
        g = np.array([(f_su(list(x + eps * e)) - f_su(list(x - eps * e))) / (2 * eps) for e in np.eye(3)])
        out[i] = -factor * (g - (x @ g) * x)
    return out


FACTOR = 1.0 / (1.2566370614359172 * 0.86)


def test_uniaxial_fourth_order_tables():
    ax = np.array([0.3, 0.4, 0.866]); ax /= np.linalg.norm(ax)
    K1, K2 = 0.5, 0.2   # simulation units (5e5 and 2e5 J/m^3)
    an = nmag.uniaxial_anisotropy(list(ax), K1=SI(K1 * 1e6, "J/m^3"), K2=SI(K2 * 1e6, "J/m^3"))
    assert an.order == 4
    T = polynomial_tables(an.function, an.order, FACTOR, quirks=None)
    m = unit_vectors(64, 1)
    E, H = eval_tables(T, m)
    a = m @ ax
    assert np.abs(E - (-K1 * a ** 2 - K2 * a ** 4)).max() < 1e-13
    g = (-2 * K1 * a - 4 * K2 * a ** 3)[:, None] * ax
    ref = -FACTOR * (g - np.sum(m * g, 1)[:, None] * m)
    assert np.abs(H - ref).max() < 1e-13 * np.abs(ref).max()
    # degree order - 1 and order + 1 monomials only
    degs = {sum((p >> s) & 15 for s in (0, 4, 8)) for p in T[2]}
    assert degs == {3, 5}


@pytest.mark.parametrize("K", [(-3e5, 0, 0), (-3e5, 1e5, 0), (2e4, 1e5, 5e4)])
def test_cubic_tables_match_tangential_gradient(K):
    # absent constants are plain zeros: an SI object is always true, so it
    # raises the order, as in the reference (anisotropy.py:190-195)
    Ks = [SI(k, "J/m^3") if k else 0 for k in K]
    cu = nmag.cubic_anisotropy([1, 0, 0], [0, 1, 0.1], K1=Ks[0], K2=Ks[1], K3=Ks[2])
    assert cu.order == (8 if K[2] else 6 if K[1] else 4)
    T = polynomial_tables(cu.function, cu.order, FACTOR, quirks=None)
    f = su_energy_function(cu.function)
    m = unit_vectors(24, 2)
    E, H = eval_tables(T, m)
    assert np.abs(E - np.array([f(list(x)) for x in m])).max() < 1e-13
    ref = fd_field(f, m, FACTOR)
    assert np.abs(H - ref).max() < 1e-8 * np.abs(ref).max()


def test_second_order_polynomial_is_the_closed_form():
    """The homogeneous degree-2 polynomial of -K1 (a.m)^2 is that expression
    itself, so its field equals the engine's closed form 2K1/(mu0 Ms)(a.m)(a -
    (a.m) m) off the unit sphere too."""
    ax = [0.0, 0.6, 0.8]
    K1 = 0.35
    an = nmag.uniaxial_anisotropy(ax, K1=SI(K1 * 1e6, "J/m^3"))
    T = polynomial_tables(an.function, 2, FACTOR, quirks=None)
    m = 1.03 * unit_vectors(32, 3)
    _, H = eval_tables(T, m)
    a = m @ np.array(ax)
    ref = 2 * K1 * FACTOR * a[:, None] * (np.array(ax) - a[:, None] * m)
    assert np.abs(H - ref).max() < 1e-14


def test_quirks_round_like_printf_f():
    cu = nmag.cubic_anisotropy([1, 1, 0], [0, 0, 1], K1=SI(4.5e4, "J/m^3"))
    T = polynomial_tables(cu.function, cu.order, FACTOR, quirks="nmag")
    for c in list(T[1]) + list(T[3]):
        assert c == float("%f" % c)
    Tx = polynomial_tables(cu.function, cu.order, FACTOR, quirks=None)
    m = unit_vectors(16, 4)
    _, H = eval_tables(T, m)
    _, Hx = eval_tables(Tx, m)
    # 6 decimals on coefficients of size ~0.1: relative error of a few 1e-6
    assert 0 < np.abs(H - Hx).max() < 1e-5 * np.abs(Hx).max() * 10


def test_fit_is_exact_for_representable_functions():
    # E = mx^2 at order 4 is mx^2 (mx^2 + my^2 + mz^2) on the sphere
    poly = dict((p, c) for c, p in spherical_polynomial(lambda m: m[0] ** 2, 4))
    assert poly == pytest.approx({(4, 0, 0): 1.0, (2, 2, 0): 1.0, (2, 0, 2): 1.0}, abs=1e-12)
    with pytest.raises(ValueError):
        spherical_polynomial(lambda m: m[0], 13)


def test_material_routing():
    ms = SI(8.6e5, "A/m")
    plain = nmag.MagMaterial("a", Ms=ms, anisotropy=nmag.uniaxial_anisotropy([0, 0, 1], K1=SI(1e5, "J/m^3")))
    c = plain.coefficients()
    assert c["anis_poly"] is None and c["K1"] == pytest.approx(0.1)
    k2 = nmag.MagMaterial("b", Ms=ms, anisotropy=nmag.uniaxial_anisotropy([0, 0, 1], K1=SI(1e5, "J/m^3"),
                                                                          K2=SI(2e4, "J/m^3")))
    c = k2.coefficients()
    assert c["K1"] == 0.0 and c["anis_coeff"] == 0.0 and len(c["anis_poly"][0]) > 0
    assert k2.anisotropy_order == 4
    # a custom energy function needs its order (main.py:416-419)
    with pytest.raises(ValueError):
        nmag.MagMaterial("c", Ms=ms, anisotropy=lambda m: SI(1e4, "J/m^3") * m[0] ** 2)
    with pytest.raises(ValueError):
        nmag.MagMaterial("c", Ms=ms, anisotropy=nmag.uniaxial_anisotropy([0, 0, 1], K1=1.0), anisotropy_order=2)
    cust = nmag.MagMaterial("c", Ms=ms, anisotropy=lambda m: SI(1e4, "J/m^3") * m[0] ** 2, anisotropy_order=2)
    e_pow, e_coef = cust.coefficients(None)["anis_poly"][:2]
    assert dict(zip(e_pow, e_coef)) == pytest.approx({pack((2, 0, 0)): 0.01})
    # sums of anisotropies (anisotropy.py:70-90)
    s = nmag.uniaxial_anisotropy([0, 0, 1], K1=SI(1e5, "J/m^3")) + nmag.cubic_anisotropy([1, 0, 0], [0, 1, 0],
                                                                                        K1=SI(1e4, "J/m^3"))
    assert s.order == 4 and not s.closed_form_uniaxial()
    x = [0.6, 0.0, 0.8]
    assert s.function(x).value == pytest.approx(-1e5 * 0.64 + 1e4 * (0.36 * 0.64))


def test_si_zero_is_neutral():
    K = SI(5e5, "J/m^3")
    assert (K - 0 * 0.5).value == 5e5 and (0 + K).value == 5e5 and (0 - K).value == -5e5
    assert (K + SI(0.0, "m")).value == 5e5
    with pytest.raises(ValueError):
        K + SI(1.0, "m")


def test_particle_batches_refuse_polynomial_anisotropy():
    from nmag import batch
    mat = nmag.MagMaterial("a", anisotropy=nmag.cubic_anisotropy([1, 0, 0], [0, 1, 0], K1=SI(1e4, "J/m^3")))
    with pytest.raises(NotImplementedError):
        batch._material_struct(mat.coefficients())


def test_anisotropy_jacobian_flag_is_accepted():
    sim = nmag.Simulation(do_anisotropy_jacobian=True)
    assert sim._do_anisotropy_jacobian


def test_oracle_evaluates_the_polynomial(small_box):
    import oracle
    mat = nmag.MagMaterial("Py", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"),
                           anisotropy=nmag.cubic_anisotropy([1, 0, 0], [0, 1, 0], K1=SI(-4e5, "J/m^3"),
                                                            K2=SI(1e5, "J/m^3")))
    c = mat.coefficients("nmag")
    om = oracle.OracleMesh(small_box.points, small_box.simplices, fill_bem=False)
    s = oracle.OracleSim(om, c, do_demag=False)
    m = unit_vectors(small_box.n_nodes, 5)
    s.rhs(m)
    E, H = eval_tables(c["anis_poly"], m)
    assert np.abs(s.field("H_anis") - H).max() < 1e-14 * np.abs(H).max()
    assert np.abs(s.energy_density(m)[3] - E).max() < 1e-14 * np.abs(E).max()
