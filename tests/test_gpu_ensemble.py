"""Ensemble form on the GPU: B simulations on one mesh in one handle
(options n_members = B), sharing every BEM pass and CG launch.  Each member
must reproduce an independent single-simulation handle."""
import numpy as np
import pytest

from conftest import permalloy, seeded_m
from test_gpu_parity import make_engine

pytestmark = pytest.mark.gpu


def make_ensemble(msh, mat, B, tol=1e-12, bem_precision=0, cg_precision=0, anchor=0.0, adjoint_cg=0,
                  anchor_product=0, jv_precision=0):
    from nmag import _lib
    single = make_engine(msh, mat, tol=tol, bem_precision=bem_precision)
    c = mat.coefficients("nmag")
    mt = _lib.Material()
    mt.Ms, mt.exch_coeff, mt.C1, mt.C2, mt.C3 = c["Ms"], c["exch_coeff"], c["C1"], c["C2"], c["C3"]
    mt.K1, mt.anis_coeff, mt.E_coeff_half, mt.E_coeff_ext = c["K1"], c["anis_coeff"], c["E_coeff_half"], c["E_coeff_ext"]
    for d in range(3):
        mt.axis[d] = c["axis"][d]
    op = _lib.Options()
    op.do_demag = 1
    op.nbc_rtol = op.dbc_rtol = tol
    op.nbc_atol = op.dbc_atol = 1e-50
    op.nbc_maxits = op.dbc_maxits = 20000
    op.bem_precision = bem_precision
    op.cg_precision = cg_precision
    op.n_members = B
    op.bem_anchor_tol = anchor
    op.adjoint_cg_precision = adjoint_cg
    op.anchor_product = anchor_product
    op.jv_precision = jv_precision
    ens = _lib.Engine(msh.points, msh.simplices, mt, op)
    if c.get("anis_poly") is not None:
        ens.set_anisotropy_poly(*c["anis_poly"])
    return ens, single


def _members(N, B, seed0=100):
    ms = np.stack([seeded_m(N, base=(1.0, 0.3 * b, -0.2), seed=seed0 + b, noise=0.5) for b in range(B)])
    hs = np.stack([np.broadcast_to([0.01 * b, -0.02, 0.005 * (b % 3)], (N, 3)) for b in range(B)])
    return ms, hs


@pytest.mark.parametrize("B,prec", [(3, 0), (10, 0), (5, 1), (1, 2), (6, 2)])
def test_ensemble_fields_match_single(cube, B, prec):
    mat = permalloy(0.5)
    ens, single = make_ensemble(cube, mat, B, bem_precision=prec)
    if prec == 2:   # the compensated form is compared with the FP64 form itself
        single = make_engine(cube, mat, bem_precision=0)
    N = len(cube.points)
    ms, hs = _members(N, max(B, 2))
    ms, hs = (ms[:B], hs[:B]) if B > 1 else (ms[0], hs[0])
    ens.set_m(ms)
    ens.set_h_ext(hs)
    f = ens.eval_fields()
    if B == 1:
        f = {k: v[None] for k, v in f.items()}
        ms, hs = ms[None], hs[None]
    assert f["H_total"].shape == (B, N, 3)
    for b in range(B):
        single.set_m(ms[b])
        single.set_h_ext(hs[b])
        g = single.eval_fields()
        # FP64 form: same operations up to summation order; FP32 form: the two
        # BEM kernels round their FP32 partial sums differently
        tol = 1e-5 if prec == 1 else 1e-9
        for k in ("H_demag", "H_total", "dmdt"):
            ref = g[k]
            assert np.abs(f[k][b] - ref).max() <= tol * np.abs(ref).max(), (b, k)
        if B > 1:
            assert np.allclose(ens.member_averages(b), single.averages(), rtol=0, atol=1e-13)
        if prec == 1:
            e = np.abs(f["H_demag"][b] - g["H_demag"]).max() / np.abs(g["H_demag"]).max()
            assert e <= 2e-6, e


def test_ensemble_integration_matches_single_runs(small_box):
    mat = permalloy(0.5)
    B = 3
    ens, single = make_ensemble(small_box, mat, B)
    N = len(small_box.points)
    ms, hs = _members(N, B, seed0=200)
    ens.set_m(ms)
    ens.set_h_ext(hs)
    ens.ts_init(0.0, rtol=1e-8, atol=1e-8)
    ens.ts_advance(5.0)
    me = ens.get_m()
    for b in range(B):
        single.set_m(ms[b])
        single.set_h_ext(hs[b])
        single.ts_init(0.0, rtol=1e-8, atol=1e-8)
        single.ts_advance(5.0)
        assert np.abs(me[b] - single.get_m()).max() <= 2e-6, b


@pytest.mark.parametrize("B", [1, 6])
def test_mixed_precision_cg_matches_fp64(cube, B):
    """FP32 CG iterations with FP64 residual refinement, refined to rtol 1e-12,
    give the FP64 CG's fields (single handle routed through the same kernel)."""
    mat = permalloy(0.5)
    ens, single = make_ensemble(cube, mat, B, cg_precision=1)
    N = len(cube.points)
    ms, hs = _members(N, max(B, 2), seed0=300)
    ens.set_m(ms[:B] if B > 1 else ms[0])
    ens.set_h_ext(hs[:B] if B > 1 else hs[0])
    f = ens.eval_fields()
    for b in range(B):
        single.set_m(ms[b])
        single.set_h_ext(hs[b])
        g = single.eval_fields()
        got = f["H_demag"][b] if B > 1 else f["H_demag"]
        ref = g["H_demag"]
        assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max(), b
