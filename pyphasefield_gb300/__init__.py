"""pyphasefield_gb300: GB300 (sm_103a) explicit time-stepping engines behind
pyphasefield's Simulation / engine plugin API.

    from pyphasefield_gb300 import Warren1995GB300
    sim = Warren1995GB300(dimensions=[1024, 1024], dx=4.6e-8,
                          boundary_conditions="NEUMANN")
    sim.initialize_fields_and_imported_data()
    sim.simulate(10000)
    sim.retrieve_fields_from_GPU()

The compute path is libppf_gb300.so (CUDA, built by
``python -m pyphasefield_gb300.build``); there is no CPU fallback.
"""
from .field import Field
from .simulation import Simulation
from .engines import (AllenCahnGB300, CahnAllenGB300, CahnHilliardGB300, DiffusionGB300,
                      NCGPUGB300, NCGPU_newGB300, Warren1995GB300, make_engines,
                      make_ncgpu, make_ncgpu_new)

__version__ = "0.1.0"
__all__ = ["Field", "Simulation", "DiffusionGB300", "CahnAllenGB300", "AllenCahnGB300",
           "CahnHilliardGB300", "Warren1995GB300", "NCGPUGB300", "NCGPU_newGB300", "make_engines",
           "make_ncgpu", "make_ncgpu_new"]
