"""GPU parity on the 500 x 125 x 3 nm film (30,753 nodes, 21,002 boundary
nodes): bit-exact CSR / boundary / triangles and the full RHS against the
oracle.  Tolerances as in test_gpu_parity.py."""
import numpy as np
import pytest

import oracle
from conftest import permalloy, seeded_m
from test_gpu_parity import make_engine, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def film_pair():
    from nmag import mesh
    film = mesh.film_mesh()
    mat = permalloy(0.02)
    eng = make_engine(film, mat, tol=1e-10)
    om = oracle.OracleMesh(film.points, film.simplices)
    return eng, om, mat


def test_film_topology_bit_exact(film_pair):
    eng, om, _ = film_pair
    assert (eng.N, eng.nnz, eng.nb, eng.nouter) == (30753, 374257, 21002, 42000)
    rp, ci, K, G, D, V = eng.csr()
    assert np.array_equal(rp, om.row_ptr) and np.array_equal(ci, om.col_idx)
    assert np.array_equal(K, om.K) and np.array_equal(G, om.G) and np.array_equal(D, om.D)
    assert np.array_equal(V, om.vol)
    nob, tri, nrm, sa = eng.boundary()
    assert np.array_equal(nob, om.node_of_b)
    assert np.array_equal(tri, om.tri) and np.array_equal(nrm, om.tri_normal)


def test_film_rhs_matches_oracle(film_pair):
    eng, om, mat = film_pair
    s = oracle.OracleSim(om, mat.coefficients("nmag"), nbc=(1e-10, 1e-50, 50000), dbc=(1e-10, 1e-50, 50000))
    m = seeded_m(om.n_nodes, base=(1.0, 0.25, 0.1), seed=1)
    eng.set_h_ext(np.zeros(3))
    eng.set_m(m)
    f = eng.eval_fields()
    d = s.rhs(m)
    assert rel_err(f["H_exch"], s.field("H_exch")) < 1e-12
    assert rel_err(f["H_demag"], s.field("H_demag")) < 1e-7
    assert rel_err(f["dmdt"], d.reshape(-1, 3)) < 1e-7
