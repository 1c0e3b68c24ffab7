"""nmg_max_dm_static: the convergence reduction for callers that may not
allocate GPU memory (programs whose device memory belongs to their own pool,
or loops that cannot afford the device-wide synchronisation of cudaMalloc).

It must give the same result as nmg_max_dm -- the entry point that allocates a
device temporary -- on two calls in a row (the static scratch is reused and
keeps the previous call's partials), and refuse sizes beyond its fixed
scratch.  Both reductions take the maximum of the same per-node values; the
tolerance is 1e-15 relative (the two kernels are compiled separately).  This file is collected last so that a
failure here cannot hide the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import permalloy, seeded_m

pytestmark = pytest.mark.gpu


def _engine(msh):
    from test_gpu_parity import make_engine
    return make_engine(msh, permalloy(0.5), do_demag=False)


def test_static_max_dm_matches_allocating_entry_point(small_box):
    import torch
    from nmag import _lib
    L = _lib.lib()
    eng = _engine(small_box)
    n = small_box.n_nodes
    for call in range(2):
        m_prev = seeded_m(n, seed=20 + call, noise=0.3)
        m_now = seeded_m(n, seed=40 + call, noise=0.3 + 0.2 * call)
        eng.set_m(m_now)
        expected = eng.max_dm(m_prev)            # allocating entry point
        d_now = torch.tensor(m_now, dtype=torch.float64, device="cuda")
        d_prev = torch.tensor(m_prev, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        out = C.c_double(-1.0)
        rc = L.nmg_max_dm_static(C.c_void_p(d_now.data_ptr()), C.c_void_p(d_prev.data_ptr()), n, C.byref(out))
        assert rc == 0, L.nmg_last_error(None)
        if call > 0:
            # the first call sets the device up (symbol lookup, module load);
            # after that a call leaves the device's free memory as it found it
            assert torch.cuda.mem_get_info()[0] == free_before
        assert out.value == pytest.approx(expected, rel=1e-15, abs=0.0)
        assert out.value == pytest.approx(np.sqrt(((m_now - m_prev) ** 2).sum(1)).max(), rel=1e-15)


def test_static_max_dm_rejects_oversized_input():
    import torch
    from nmag import _lib
    L = _lib.lib()
    d = torch.zeros(3, dtype=torch.float64, device="cuda")
    out = C.c_double(-1.0)
    rc = L.nmg_max_dm_static(C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), 2097152 + 1, C.byref(out))
    assert rc == -2
    assert b"static scratch limit" in L.nmg_last_error(None)
    assert out.value == -1.0
