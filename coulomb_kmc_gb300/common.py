"""Shared definitions mirroring coulomb_kmc/common.py."""
from enum import Enum

import numpy as np


class BCType(Enum):
    """Boundary condition type (coulomb_kmc/common.py:37-50)."""
    PBC = "pbc"
    FREE_SPACE = "free_space"
    NEAREST = "27"
    FF_ONLY = "ff-only"


def spherical(xyz):
    """(radius, polar angle, longitude) of cartesian points (coulomb_kmc/common.py:6-34)."""
    if isinstance(xyz, tuple):
        x, y, z = xyz
        xy = x * x + y * y
        return np.array((np.sqrt(xy + z * z), np.arctan2(np.sqrt(xy), z), np.arctan2(y, x)))
    xyz = np.atleast_2d(xyz)
    out = np.zeros(xyz.shape)
    xy = xyz[:, 0] ** 2 + xyz[:, 1] ** 2
    out[:, 0] = np.sqrt(xy + xyz[:, 2] ** 2)
    out[:, 1] = np.arctan2(np.sqrt(xy), xyz[:, 2])
    out[:, 2] = np.arctan2(xyz[:, 1], xyz[:, 0])
    return out


# the 27 neighbour offsets, x fastest (coulomb_kmc/common.py:53-81)
cell_offsets = tuple((x, y, z) for z in (-1, 0, 1) for y in (-1, 0, 1) for x in (-1, 0, 1))
cell_offsets_26 = tuple(o for o in cell_offsets if o != (0, 0, 0))
