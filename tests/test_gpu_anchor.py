"""Anchored compensated BEM product (bem_anchor_tol): B x is formed as
B x0 + B32 (x - x0) from the last compensated product (x0, B x0) while x
stays within tol of x0 (max norm, per member).  Checked against the FP64
form at the same magnetisation, with the anchor's refresh decisions read
back from the library's counters."""
import numpy as np
import pytest

from conftest import permalloy, seeded_m
from test_gpu_ensemble import make_ensemble

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("B", [1, 3, 10])
def test_anchor_refresh_decisions_and_accuracy(cube, B):
    mat = permalloy(0.5)
    anc, _ = make_ensemble(cube, mat, B, bem_precision=2, anchor=0.02)
    ref, _ = make_ensemble(cube, mat, B, bem_precision=0)
    N = len(cube.points)
    shape = (B, N, 3) if B > 1 else (N, 3)
    ms = np.stack([seeded_m(N, base=(1.0, 0.2 * b, -0.3), seed=300 + b, noise=0.5) for b in range(B)]).reshape(shape)
    hs = np.broadcast_to([0.02, -0.01, 0.005], shape).copy()
    for e in (anc, ref):
        e.set_h_ext(hs)
    chunks = (B + 7) // 8
    rng = np.random.default_rng(7)

    def step(m):
        anc.set_m(m)
        ref.set_m(m)
        return anc.eval_fields(), ref.eval_fields()

    # 1: no anchor yet -> every chunk refreshes (compensated product)
    f, g = step(ms)
    assert anc.bem_anchor_stats() == (chunks, chunks)
    assert _rel(f["H_demag"], g["H_demag"]) <= 1e-9
    # 2: a small move (drift well inside tol) -> the FP32 difference product
    m2 = ms + 2e-4 * rng.standard_normal(ms.shape)
    m2 /= np.linalg.norm(m2, axis=-1, keepdims=True)
    f, g = step(m2)
    assert anc.bem_anchor_stats() == (2 * chunks, chunks)
    assert _rel(f["H_demag"], g["H_demag"]) <= 1e-9
    assert _rel(f["H_total"], g["H_total"]) <= 1e-9
    # 3: a large move (a new magnetisation) -> refresh again
    m3 = np.stack([seeded_m(N, base=(-0.4, 1.0, 0.1 * b), seed=400 + b, noise=0.5) for b in range(B)]).reshape(shape)
    f, g = step(m3)
    assert anc.bem_anchor_stats() == (3 * chunks, 2 * chunks)
    assert _rel(f["H_demag"], g["H_demag"]) <= 1e-9
    anc.close()
    ref.close()


def test_anchor_difference_algebra(cube):
    """A huge tol: after the first product every product is anchored however
    far x moves, so the result carries the FP32 product error of the full
    difference x - x0 (here about twice |x|), bounded like the FP32 form's."""
    mat = permalloy(0.5)
    B = 2
    anc, _ = make_ensemble(cube, mat, B, bem_precision=2, anchor=1e6)
    ref, _ = make_ensemble(cube, mat, B, bem_precision=0)
    N = len(cube.points)
    ma = np.stack([seeded_m(N, base=(1.0, 0.0, 0.0), seed=500 + b, noise=0.3) for b in range(B)])
    mb = np.stack([seeded_m(N, base=(0.0, 1.0, 0.5), seed=600 + b, noise=0.3) for b in range(B)])
    hs = np.zeros((B, N, 3))
    for e in (anc, ref):
        e.set_h_ext(hs)
    anc.set_m(ma)
    anc.eval_fields()
    anc.set_m(mb)
    ref.set_m(mb)
    f, g = anc.eval_fields(), ref.eval_fields()
    assert anc.bem_anchor_stats() == (2, 1)
    assert _rel(f["H_demag"], g["H_demag"]) <= 5e-6   # the FP32 form's bound on this mesh, x2
    anc.close()
    ref.close()


def test_anchor_suspended_on_rk4_tape(cube):
    """The RK4 tape recomputes segments bit for bit, so its runs bypass the
    anchor: the counters do not move and two runs agree exactly."""
    from test_gpu_adjoint import _params, _run
    mat = permalloy(0.5)
    eng, _ = make_ensemble(cube, mat, 1, bem_precision=2, anchor=0.02)
    c = mat.coefficients("nmag")
    N, T = len(cube.points), len(cube.simplices)
    eng.set_h_ext(np.zeros(3))
    m0 = seeded_m(N, seed=11)
    Ms_T, K1_T, pulses = _params(T, 2)
    a = _run(eng, c, m0, Ms_T, K1_T, pulses, 6, 2, 3)
    b = _run(eng, c, m0, Ms_T, K1_T, pulses, 6, 2, 3)
    assert eng.bem_anchor_stats() == (0, 0)
    assert a[0] == b[0]
    for x, y in zip(a[1:], b[1:]):
        assert np.array_equal(x, y)
    eng.clear_element_params()
    eng.close()


def test_anchored_ensemble_integration_matches_fp64(small_box):
    """A joint BDF run of 3 members through the chosen form (compensated
    product anchored at 3e-3, FP32 CG with FP64 refinement) follows the FP64
    form's trajectories; most products are anchored differences."""
    mat = permalloy(0.5)
    B = 3
    anc, _ = make_ensemble(small_box, mat, B, bem_precision=2, cg_precision=1, anchor=3e-3)
    ref, _ = make_ensemble(small_box, mat, B, bem_precision=0)
    N = len(small_box.points)
    ms = np.stack([seeded_m(N, base=(1.0, 0.3 * b, -0.2), seed=700 + b, noise=0.5) for b in range(B)])
    hs = np.stack([np.broadcast_to([0.01 * b, -0.02, 0.005], (N, 3)) for b in range(B)])
    for e in (anc, ref):
        e.set_m(ms)
        e.set_h_ext(hs)
        e.ts_init(0.0, rtol=1e-8, atol=1e-8)
        e.ts_advance(5.0)
    prod, refr = anc.bem_anchor_stats()
    assert prod > 20 and refr < prod // 2, (prod, refr)
    assert np.abs(anc.get_m() - ref.get_m()).max() <= 2e-6
    anc.close()
    ref.close()


def test_fp16_fragment_difference_product(cube):
    """anchor_product 1: the difference B (x - x0) of the anchored ensemble
    product from the FP16 fragment copy of B on the tensor cores
    (mma.m16n8k16, FP32 accumulation).  Ten members (a chunk of 8 and one of
    2, so unused operand columns are exercised).  A refresh is the
    compensated product itself; after a small move the result stays within
    FP16 rounding of |B||x - x0| of the FP32-difference form, and a wrong
    fragment order would be off by O(1)."""
    mat = permalloy(0.5)
    B = 10
    h16, _ = make_ensemble(cube, mat, B, bem_precision=2, anchor=0.02, anchor_product=1)
    f32, _ = make_ensemble(cube, mat, B, bem_precision=2, anchor=0.02, anchor_product=0)
    ref, _ = make_ensemble(cube, mat, B, bem_precision=0)
    N = len(cube.points)
    ms = np.stack([seeded_m(N, base=(1.0, 0.2 * b, -0.3), seed=700 + b, noise=0.5) for b in range(B)])
    hs = np.broadcast_to([0.02, -0.01, 0.005], (B, N, 3)).copy()
    for e in (h16, f32, ref):
        e.set_h_ext(hs)
        e.set_m(ms)
    f, g = h16.eval_fields(), ref.eval_fields()
    assert h16.bem_anchor_stats() == (2, 2)
    assert _rel(f["H_demag"], g["H_demag"]) <= 1e-9          # refresh: the compensated product
    f32.eval_fields()
    rng = np.random.default_rng(8)
    m2 = ms + 1e-3 * rng.standard_normal(ms.shape)
    m2 /= np.linalg.norm(m2, axis=-1, keepdims=True)
    for e in (h16, f32, ref):
        e.set_m(m2)
    f, f3, g = h16.eval_fields(), f32.eval_fields(), ref.eval_fields()
    assert h16.bem_anchor_stats() == (4, 2)                   # both chunks anchored
    e16 = _rel(f["H_demag"], g["H_demag"])
    assert _rel(f3["H_demag"], g["H_demag"]) <= 1e-9
    assert e16 <= 2e-5, e16
    for b in range(B):                                        # every member, both chunks
        assert _rel(f["H_demag"][b], g["H_demag"][b]) <= 2e-5, b
    h16.close()
    f32.close()
    ref.close()
