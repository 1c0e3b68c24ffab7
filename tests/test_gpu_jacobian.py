"""The Newton matrix's Jacobian levels (nmg_set_jacobian) against finite
differences of the right-hand side, and the BDF trajectory with the exact
Jacobian against the oracle.

J(m) v from nmg_jacobian_apply is compared with the central difference
(f(m + e v) - f(m - e v)) / 2e of nmg_rhs_device, both with Poisson solves at
1e-12 (e = 1e-4: the difference's truncation error e^2 |f'''| / 6 and its
rounding error ~1e-16 |f| / e stay near 1e-8 of |J v|).  The directions are
smooth fields (a long-wavelength rotation of m), for which the exchange part
does not swamp the others:

* level 2 ("exact") agrees with the difference to 1e-6 of max |J v|;
* level 0 (the reference's Jacobian: exchange only) misses the demag,
  anisotropy and C3 terms, by more than 1e-2 here;
* level 1 ("local") misses only the demag response: exact without demag.

The reference's Jacobian is approximate by design (nmag_lam.py:665-704), so
the trajectory with the exact one agrees with the oracle's (approximate J)
to the integrators' tolerance, like the default's (1e-4 over 300 ps).
"""
import numpy as np
import pytest

import nmag
from nmag import SI
from conftest import permalloy, seeded_m
from test_gpu_parity import make_engine

pytestmark = pytest.mark.gpu

EPS = 1e-4
TOL_EXACT = 1e-6


def anis_material(alpha=0.5):
    return nmag.MagMaterial("Co", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=alpha,
                            llg_gamma_G=SI(2.211e5, "m/A s"),
                            anisotropy=nmag.uniaxial_anisotropy([0.3, 0.2, 1.0], K1=SI(5e5, "J/m^3")))


def smooth_direction(points, m, seed):
    """A smooth tangent-ish direction: m rotated about a random axis with a
    long-wavelength angle field, plus a small length change (so the C3 term's
    derivative is exercised)."""
    rng = np.random.default_rng(seed)
    ext = points.max(0) - points.min(0)
    k = rng.uniform(0.5, 1.5, size=3) * np.pi / np.maximum(ext, 1e-30)
    ang = np.sin(points @ k + rng.uniform(0, np.pi))
    ax = rng.standard_normal(3)
    ax /= np.linalg.norm(ax)
    return ang[:, None] * np.cross(ax, m) + 0.05 * np.cos(points @ (0.7 * k))[:, None] * m


def _dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def jv(eng, m, v):
    import torch
    dm, dv = _dev(m), _dev(v)
    out = torch.empty_like(dm)
    torch.cuda.synchronize()
    eng.jacobian_apply_device(dm.data_ptr(), dv.data_ptr(), out.data_ptr())
    return out.cpu().numpy()


def rhs(eng, m):
    import torch
    dm = _dev(m)
    out = torch.empty_like(dm)
    torch.cuda.synchronize()
    eng.rhs_device(dm.data_ptr(), out.data_ptr())
    return out.cpu().numpy()


def fd(eng, m, v, e=EPS):
    return (rhs(eng, m + e * v) - rhs(eng, m - e * v)) / (2.0 * e)


def errors(eng, m, v):
    ref = fd(eng, m, v)
    scale = np.abs(ref).max()
    out = {}
    for level, name in enumerate(("approximate", "local", "exact")):
        eng.set_jacobian(level, 1e-12)
        out[name] = np.abs(jv(eng, m, v) - ref).max() / scale
    return out


@pytest.mark.parametrize("seed", [0, 1])
def test_exact_jacobian_matches_finite_differences(cube, seed):
    eng = make_engine(cube, anis_material(), tol=1e-12)
    N = len(cube.points)
    m = seeded_m(N, base=(1.0, 0.3, 0.5), seed=10 + seed, noise=0.2)
    eng.set_h_ext(np.array([0.05, -0.02, 0.01]))
    v = smooth_direction(cube.points, m, seed)
    err = errors(eng, m, v)
    print("cube, uniaxial K1 + demag, direction %d: J v against the difference %s" % (seed, err))
    assert err["exact"] <= TOL_EXACT, err
    assert err["approximate"] > 1e-2, err
    assert err["local"] > 1e-3, err   # the demag response is not small for a smooth direction
    eng.close()


def test_local_jacobian_is_exact_without_demag(cube):
    from test_gpu_anisotropy import cubic_material
    for mat in (anis_material(), cubic_material()):   # uniaxial K1 and a polynomial (cubic K1-K3) table
        eng = make_engine(cube, mat, do_demag=False, tol=1e-12)
        N = len(cube.points)
        m = seeded_m(N, base=(0.4, 1.0, 0.2), seed=3, noise=0.3)
        eng.set_h_ext(np.zeros(3))
        v = smooth_direction(cube.points, m, 5)
        err = errors(eng, m, v)
        print("cube without demag, %s: %s" % (mat.name, err))
        assert err["local"] <= TOL_EXACT, err
        assert err["exact"] <= TOL_EXACT, err
        assert err["approximate"] > 1e-3, err
        eng.close()


def test_exact_jacobian_ensemble_members(cube):
    """Three members in one handle: each member's J v equals the one-member
    handle's for the same state and direction (the demag response of all
    members from one batched pipeline)."""
    from test_gpu_ensemble import make_ensemble
    B = 3
    ens, single = make_ensemble(cube, anis_material(), B, tol=1e-12)
    N = len(cube.points)
    ms = np.stack([seeded_m(N, base=(1.0, 0.2 * b, -0.3), seed=40 + b, noise=0.3) for b in range(B)])
    vs = np.stack([smooth_direction(cube.points, ms[b], 20 + b) for b in range(B)])
    for e in (ens, single):
        e.set_h_ext(np.zeros(3))
        e.set_jacobian(2, 1e-12)
    got = jv(ens, ms, vs).reshape(B, N, 3)
    for b in range(B):
        ref = jv(single, ms[b], vs[b])
        err = np.abs(got[b] - ref).max() / np.abs(ref).max()
        print("ensemble member %d: J v against one member %.2e" % (b, err))
        assert err <= 1e-8, (b, err)
    ens.close()
    single.close()


def test_exact_jacobian_several_materials():
    """Two materials on shared nodes with local couplings and a uniaxial
    anisotropy on one: level 2 against the difference on the site vector."""
    from test_gpu_multimat import engine, halves, materials
    msh = halves()
    py, co = materials()
    eng = engine(msh, [[0, 1], [1]], [py, co])
    eng.set_local_coupling(0, 1, -0.3, -0.12)
    eng.set_local_coupling(1, 0, -0.2, -0.08)
    site_node, _ = eng.site_info()
    pts = msh.points[site_node]
    m = seeded_m(len(site_node), base=(0.2, 1.0, 0.4), seed=7, noise=0.3)
    eng.set_h_ext(np.array([0.01, 0.0, -0.02]))
    v = smooth_direction(pts, m, 9)
    err = errors(eng, m, v)
    print("two materials with local couplings: %s" % err)
    assert err["exact"] <= TOL_EXACT, err
    assert err["approximate"] > 1e-3, err
    eng.close()


def test_exact_jacobian_trajectory_matches_oracle(cube):
    """The cube with uniaxial anisotropy, alpha 0.5, 300 ps: the BDF with
    each Jacobian level against the oracle's BDF (approximate Jacobian), m(t)
    every 10 ps within 1e-4; the Newton iteration counts are printed."""
    import oracle
    from test_gpu_trajectory import _oracle_run
    mat = anis_material(0.5)
    om = oracle.OracleMesh(cube.points, cube.simplices)
    m0 = seeded_m(om.n_nodes, base=(1.0, 0.6, -0.4), seed=2, noise=0.05)
    h = np.array([0.02, 0.0, 0.0])
    times = [10.0 * k for k in range(1, 31)]
    mo, _, so = _oracle_run(om, mat, m0, h, times, 1e-10)
    eng = make_engine(cube, mat, tol=1e-10)
    for level in (0, 1, 2):
        eng.set_jacobian(level, 1e-6)
        eng.set_h_ext(h)
        eng.set_m(m0)
        eng.ts_init(0.0, 1e-6, 1e-6, 2, 300)
        dm = []
        for k, t in enumerate(times):
            _, st = eng.ts_advance(t)
            dm.append(np.abs(eng.get_m() - mo[k]).max())
        print("jacobian level %d: max |dm| %.2e over 300 ps; steps %d, Newton %d, Krylov %d, "
              "convergence failures %d, RHS %d (oracle: %d steps, %d Newton)"
              % (level, max(dm), st["nst"], st["nni"], st["nli"], st["ncfn"], st["nfe"], so["nst"], so["nni"]))
        assert max(dm) <= 1e-4, (level, max(dm))
    assert np.abs(mo[-1] - m0).max() > 1e-2   # the state moved
    eng.close()


def test_simulation_exact_jacobian_option(cube):
    """Simulation(jacobian="exact") relaxes to the same state as the default."""
    from nmag import mesh as nmesh
    finals = []
    for jac in ("approximate", "exact"):
        sim = nmag.Simulation("jac_" + jac, jacobian=jac, jacobian_demag_rtol=1e-6)
        sim.load_mesh(nmesh.cube_mesh(), [("cube", anis_material(1.0))], unit_length=SI(1e-9, "m"))
        sim.set_m([1.0, 0.7, -0.2])
        sim.advance_time(SI(50e-12, "s"))
        finals.append(np.asarray(sim.get_subfield("m_Co")))
    d = np.abs(finals[0] - finals[1]).max()
    print("Simulation after 50 ps, approximate against exact Jacobian: max |dm| %.2e" % d)
    assert d <= 1e-4


def test_fp32_jacobian_products_match_fp64(cube):
    """jv_precision 1: the approximate Jacobian's products in FP32 arithmetic
    against the FP64 ones, for a smooth and a rough direction (relative to
    max |J v|: FP32 rounding of ~15-term sums, 1e-5); one member and an
    ensemble of three."""
    from test_gpu_ensemble import make_ensemble
    N = len(cube.points)
    rng = np.random.default_rng(4)
    for B in (1, 3):
        engs = []
        for prec in (0, 1):
            if B == 1:
                e = make_engine(cube, anis_material(), tol=1e-12, jv_precision=prec)
            else:
                e, single = make_ensemble(cube, anis_material(), B, tol=1e-12, jv_precision=prec)
                single.close()
            e.set_h_ext(np.array([0.02, 0.0, -0.01]))
            engs.append(e)
        ms = np.stack([seeded_m(N, base=(1.0, 0.3, 0.5), seed=60 + b, noise=0.2) for b in range(B)])
        for kind in ("smooth", "rough"):
            if kind == "smooth":
                vs = np.stack([smooth_direction(cube.points, ms[b], 70 + b) for b in range(B)])
            else:
                vs = rng.standard_normal((B, N, 3))
            m_in, v_in = (ms[0], vs[0]) if B == 1 else (ms, vs)
            ref, got = jv(engs[0], m_in, v_in), jv(engs[1], m_in, v_in)
            err = np.abs(got - ref).max() / np.abs(ref).max()
            print("FP32 J v, %d member(s), %s direction: %.2e of max |J v|" % (B, kind, err))
            assert err <= 1e-5, (B, kind, err)
        for e in engs:
            e.close()


def test_fp32_jacobian_trajectory_matches_oracle(cube):
    """The BDF with FP32 Jacobian-vector products: m(t) of the cube (uniaxial
    anisotropy, alpha 0.5) every 10 ps over 300 ps against the oracle's BDF
    within 1e-4, and the Newton / Krylov counts beside the FP64 form's."""
    import oracle
    from test_gpu_trajectory import _oracle_run
    mat = anis_material(0.5)
    om = oracle.OracleMesh(cube.points, cube.simplices)
    m0 = seeded_m(om.n_nodes, base=(1.0, 0.6, -0.4), seed=2, noise=0.05)
    h = np.array([0.02, 0.0, 0.0])
    times = [10.0 * k for k in range(1, 31)]
    mo, _, so = _oracle_run(om, mat, m0, h, times, 1e-10)
    for prec in (0, 1):
        eng = make_engine(cube, mat, tol=1e-10, jv_precision=prec)
        eng.set_h_ext(h)
        eng.set_m(m0)
        eng.ts_init(0.0, 1e-6, 1e-6, 2, 300)
        dm = []
        for k, t in enumerate(times):
            _, st = eng.ts_advance(t)
            dm.append(np.abs(eng.get_m() - mo[k]).max())
        print("jv_precision %d: max |dm| %.2e over 300 ps; steps %d, Newton %d, Krylov %d, convergence failures %d"
              % (prec, max(dm), st["nst"], st["nni"], st["nli"], st["ncfn"]))
        assert max(dm) <= 1e-4, (prec, max(dm))
        eng.close()
