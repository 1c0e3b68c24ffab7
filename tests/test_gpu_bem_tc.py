"""The tensor-core BEM product (bem_precision 3) against FP64.

B and each right-hand side are split into three BF16 planes; six tcgen05
products per term with FP32 sums over at most 2048 terms, added in FP64.
The split keeps ~24 significant bits of each operand; the tensor cores'
FP32 accumulation (about a thousand MMA accumulations per split and
accumulator) sets the error, so the product is compared with the FP64
product B x (numpy, from the device's own FP64 matrix) relative to |B||x| at
2e-6, and the fields of an ensemble whose members all go through one
tensor-core product with the FP64 ensemble's at the metric's 1e-5.
"""
import numpy as np
import pytest

from conftest import permalloy, seeded_m
from test_gpu_parity import make_engine

pytestmark = pytest.mark.gpu

TOL_PRODUCT = 2e-6


def _apply(eng, X):
    import torch
    dx = torch.tensor(np.ascontiguousarray(X), dtype=torch.float64, device="cuda")
    dy = torch.empty_like(dx)
    torch.cuda.synchronize()
    eng.bem_apply_device(dx.data_ptr(), dy.data_ptr(), X.shape[0])
    return dy.cpu().numpy()


def _check(B, X, Y):
    ref = X @ B.T                      # y_n = B x_n, member-major rows
    scale = (np.abs(X) @ np.abs(B).T).max()
    return np.abs(Y - ref).max() / scale


@pytest.mark.parametrize("R", [1, 5, 33, 100, 130])
def test_tc_product_matches_fp64(cube, R):
    eng = make_engine(cube, permalloy(0.5), bem_precision=3)
    B = eng.bem()
    rng = np.random.default_rng(R)
    # right-hand sides of very different scales, and one smooth (a potential-like) vector
    X = rng.standard_normal((R, eng.nb)) * (10.0 ** rng.uniform(-3, 3, size=(R, 1)))
    X[0] = np.sin(np.arange(eng.nb) * 0.01) * 100.0
    for call in range(2):   # the second call reuses the planes and buffers
        err = _check(B, X, _apply(eng, X))
        print("tensor-core product, R = %d, call %d: %.2e of max |B||x|" % (R, call, err))
        assert err <= TOL_PRODUCT, (R, call, err)
    eng.close()


def test_tc_product_tile_widths_in_one_handle(cube):
    """Calls with R needing 32-, 64- and 128-wide tiles in turn, then a small
    one again: the buffers and tensor maps follow, the results stay exact."""
    eng = make_engine(cube, permalloy(0.5), bem_precision=3)
    B = eng.bem()
    rng = np.random.default_rng(5)
    for R in (20, 60, 120, 3, 64, 7):
        X = rng.standard_normal((R, eng.nb))
        assert _check(B, X, _apply(eng, X)) <= TOL_PRODUCT, R
    eng.close()


@pytest.mark.parametrize("Bm", [1, 20])
def test_tc_ensemble_fields_match_fp64(cube, Bm):
    from test_gpu_ensemble import make_ensemble
    mat = permalloy(0.5)
    tc, _ = make_ensemble(cube, mat, Bm, bem_precision=3)
    ref, _ = make_ensemble(cube, mat, Bm, bem_precision=0)
    N = len(cube.points)
    ms = np.stack([seeded_m(N, base=(1.0, 0.2 * b, -0.3), seed=500 + b, noise=0.5) for b in range(Bm)])
    ms = ms.reshape((Bm, N, 3) if Bm > 1 else (N, 3))
    for e in (tc, ref):
        e.set_h_ext(np.zeros(3))
        e.set_m(ms)
    f, g = tc.eval_fields(), ref.eval_fields()
    for key in ("H_demag", "H_total", "dmdt"):
        err = np.abs(f[key] - g[key]).max() / np.abs(g[key]).max()
        print("tensor-core ensemble of %d: %s %.2e" % (Bm, key, err))
        assert err <= 1e-5, (key, err)
    tc.close()
    ref.close()


def test_tc_product_on_the_film():
    """The film's 21,002-node boundary: smooth potentials through the
    product, against the FP64 form; then the fields of random magnetisations
    (the 1,000-field precision configuration's kind, exchange-dominated)
    within the metric's 1e-5.  A single product at FP32-level accuracy is
    not enough on a smooth film state, where phi1 + phi2 cancels ~50-fold
    (the same limit as the FP32 form): there the error is only bounded
    loosely here, and the chosen form keeps its compensated anchor."""
    from nmag import mesh
    film = mesh.film_mesh()
    eng = make_engine(film, permalloy(0.02), tol=1e-10, bem_precision=3)
    ref = make_engine(film, permalloy(0.02), tol=1e-10, bem_precision=0)
    # smooth boundary potentials (|B x| comparable to |B||x|) of different wavelengths
    k = np.arange(eng.nb)
    X = np.stack([100.0 * np.sin(k * w + ph) for w, ph in zip(np.geomspace(1e-4, 1e-1, 8), range(8))])
    Y, Yr = _apply(eng, X), _apply(ref, X)
    err = np.abs(Y - Yr).max() / np.abs(Yr).max()
    print("tensor-core product on the film: %.2e of max |B x|" % err)
    assert err <= 1e-5, err
    for seed in (100, 101):
        g = np.random.default_rng(seed).standard_normal((eng.N, 3))
        m = g / np.linalg.norm(g, axis=1)[:, None]
        for e in (eng, ref):
            e.set_h_ext(np.zeros(3))
            e.set_m(m)
        f, h = eng.eval_fields(), ref.eval_fields()
        err_h = np.abs(f["H_total"] - h["H_total"]).max() / np.abs(h["H_total"]).max()
        print("tensor-core form on the film, random field %d: H_total %.2e" % (seed, err_h))
        assert err_h <= 1e-5, err_h
    m = seeded_m(eng.N, base=(1.0, 0.25, 0.1), seed=1)
    for e in (eng, ref):
        e.set_m(m)
    f, h = eng.eval_fields(), ref.eval_fields()
    err_s = np.abs(f["H_total"] - h["H_total"]).max() / np.abs(h["H_total"]).max()
    print("tensor-core form on the film, smooth seeded state: H_total %.2e" % err_s)
    assert err_s <= 1e-3, err_s
    eng.close()
    ref.close()
