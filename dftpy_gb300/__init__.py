"""GB300-native (sm_103a) orbital-free DFT hot path with the call surfaces of
DFTpy (Quantum-MultiScale/DFTpy): functionals, fields, grids, Ewald and the
density optimiser, evaluated by the in-tree CUDA library ``libofdft.so``
through its C ABI (include/ofdft.h)."""
from . import _lib
from .constants import BOHR, C_TF, HARTREE, ZERO
from .ewald import ewald
from .field import DirectField, ReciprocalField
from .functional import (KEDF, XC, Functional, FunctionalOutput, Hartree, LocalPseudo, TotalFunctional,
                         read_recpot, write_recpot)
from .grid import DirectGrid, ReciprocalGrid
from .ions import Ions
from .optimization import Optimization

__version__ = "0.1.0"

__all__ = ["DirectGrid", "ReciprocalGrid", "DirectField", "ReciprocalField", "Functional", "FunctionalOutput",
           "TotalFunctional", "KEDF", "XC", "Hartree", "LocalPseudo", "ewald", "Ions", "Optimization",
           "read_recpot", "write_recpot", "BOHR", "HARTREE", "C_TF", "ZERO", "load_library"]


def load_library():
    """Load (building with nvcc if needed) the native library; returns the ctypes handle."""
    return _lib.load()
