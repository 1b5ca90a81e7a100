"""GB300 engines, exported like the reference's Engines package
(Engines/__init__.py:8-23 exports every class of every engine module)."""
from .models import (AllenCahnGB300, CahnAllenGB300, CahnHilliardGB300, DiffusionGB300,
                     Warren1995GB300, make_engines)
from .ncgpu import NCGPU_newGB300, NCGPUGB300, make_ncgpu, make_ncgpu_new

__all__ = ["DiffusionGB300", "CahnAllenGB300", "AllenCahnGB300", "CahnHilliardGB300",
           "Warren1995GB300", "NCGPUGB300", "NCGPU_newGB300", "make_engines",
           "make_ncgpu", "make_ncgpu_new"]
