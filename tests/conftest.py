"""Shared test setup: import paths, the ``gpu`` marker and common fixtures.

Tests marked ``gpu`` run the CUDA library on a GB300 and compare it with the
CPU oracle (oracle/, test infrastructure only).  Everything else runs on CPU.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "nmag-src_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a library")


def permalloy(alpha=0.5, gamma=2.211e5):
    import nmag
    from nmag import SI
    return nmag.MagMaterial("Py", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=alpha,
                            llg_gamma_G=SI(gamma, "m/A s"))


def seeded_m(n_nodes, base=(1.0, 1.0, 1.0), seed=0, noise=0.01):
    rng = np.random.default_rng(seed)
    m = np.asarray(base, dtype=np.float64)[None, :] + noise * rng.standard_normal((n_nodes, 3))
    return m / np.linalg.norm(m, axis=1)[:, None]


@pytest.fixture(scope="session")
def cube():
    from nmag import mesh
    return mesh.cube_mesh()


@pytest.fixture(scope="session")
def small_box():
    from nmag import mesh
    return mesh.box_mesh(4, 3, 2, 2.0, 2.5, 1.5)
