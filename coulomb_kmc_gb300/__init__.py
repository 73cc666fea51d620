"""GB300-native FMM-KMC energy-difference path (drop-in for coulomb_kmc.KMCFMM)."""
from .common import BCType, cell_offsets, spherical
from .kmc_fmm import KMCFMM
from . import dats, lattice

__all__ = ["KMCFMM", "BCType", "cell_offsets", "spherical", "dats", "lattice"]
