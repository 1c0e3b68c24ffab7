"""nmag (GB300 build): the LLG right-hand side and time integration of
nmag/nsim on hand-written sm_103a CUDA kernels, behind nmag's Python API.

    import nmag
    from nmag import SI
    mat = nmag.MagMaterial("Py", Ms=SI(0.86e6, "A/m"), exchange_coupling=SI(13e-12, "J/m"), llg_damping=0.5)
    sim = nmag.Simulation()
    sim.load_mesh(nmag.mesh.cube_mesh(), [("cube", mat)], unit_length=SI(1e-9, "m"))
    sim.set_m([1, 1, 1])
    sim.advance_time(SI(1e-12, "s"))
"""
from . import mesh
from .si import SI, simulation_units
from .material import MagMaterial
from .anisotropy import PredefinedAnisotropy, uniaxial_anisotropy, cubic_anisotropy
from .simulation import Simulation, every, at, never
from .sets import float_set, vector_set
from .vectools import normalised_vector, vector3_dot, vector3_cross
from ._lib import NmagGpuError
from .h5data import (get_subfield_from_h5file, get_subfield_positions_from_h5file,
                     get_subfield_sites_from_h5file)

__all__ = ["SI", "simulation_units", "MagMaterial", "PredefinedAnisotropy", "uniaxial_anisotropy", "cubic_anisotropy",
           "Simulation", "every", "at", "never", "mesh",
           "float_set", "vector_set", "normalised_vector", "vector3_dot", "vector3_cross", "NmagGpuError",
           "get_subfield_from_h5file", "get_subfield_positions_from_h5file", "get_subfield_sites_from_h5file"]
