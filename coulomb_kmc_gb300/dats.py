"""Minimal stand-ins for the ppmd data model used by the KMCFMM interface.

The reference takes ppmd ``PositionDat`` / ``ParticleDat`` / ``ScalarArray``
objects and a domain with an ``extent`` (coulomb_kmc/kmc_fmm.py:436-451,
:665-704).  ppmd is not a dependency here; these classes provide the pieces of
that surface the KMC path touches (``.data``, ``.view``, ``[]``, ``.ncomp``,
``.dtype``, ``.npart_local``, ``.group``, ``.modify_view()``, ``domain.extent``).
Plain numpy arrays and torch tensors are accepted wherever a dat is.
"""
import contextlib
import ctypes

import numpy as np

REAL = ctypes.c_double
INT64 = ctypes.c_int64

_NP = {ctypes.c_double: np.float64, ctypes.c_int64: np.int64, np.float64: np.float64, np.int64: np.int64,
       float: np.float64, int: np.int64}


class Domain:
    """Cubic simulation domain [-E/2, E/2]^3 (ppmd BaseDomainHalo's ``extent``)."""

    def __init__(self, extent):
        e = np.atleast_1d(np.asarray(extent, dtype=np.float64))
        if e.size == 1:
            e = np.repeat(e, 3)
        self.extent = e
        self.comm = None


class State:
    """Holder of dats that share a particle count and a domain (ppmd ``State``)."""

    def __init__(self, domain=None, npart=0):
        self.domain = domain
        self.npart = npart

    @property
    def npart_local(self):
        return self.npart


class ParticleDat:
    """Per-particle array of shape (npart, ncomp)."""

    def __init__(self, npart=0, ncomp=1, dtype=REAL, group=None, initial_value=None):
        self.ncomp = int(ncomp)
        self.dtype = dtype
        self.data = np.zeros((int(npart), self.ncomp), dtype=_NP.get(dtype, dtype))
        if initial_value is not None:
            self.data[:] = initial_value
        self.group = group

    @property
    def view(self):
        return self.data

    @property
    def npart_local(self):
        return self.data.shape[0]

    def __getitem__(self, key):
        return self.data[key]

    def __setitem__(self, key, value):
        self.data[key] = value

    @contextlib.contextmanager
    def modify_view(self):
        yield self.data


class PositionDat(ParticleDat):
    """Per-particle positions, shape (npart, 3)."""

    def __init__(self, npart=0, group=None, initial_value=None):
        super().__init__(npart, 3, REAL, group, initial_value)


class ScalarArray:
    """Small global array (ppmd ``ScalarArray``)."""

    def __init__(self, initial_value=None, ncomp=1, dtype=REAL):
        if initial_value is not None:
            self.data = np.array(initial_value, dtype=_NP.get(dtype, dtype)).ravel()
        else:
            self.data = np.zeros(int(ncomp), dtype=_NP.get(dtype, dtype))
        self.ncomp = self.data.size
        self.dtype = dtype

    @property
    def view(self):
        return self.data

    def __getitem__(self, key):
        return self.data[key]

    def __setitem__(self, key, value):
        self.data[key] = value


def make_state(positions, charges, extent):
    """Convenience: a State with a PositionDat ``P`` and a charge ParticleDat ``Q``."""
    positions = np.asarray(positions, dtype=np.float64)
    n = positions.shape[0]
    st = State(Domain(extent), n)
    st.P = PositionDat(n, group=st, initial_value=positions)
    st.Q = ParticleDat(n, 1, REAL, group=st, initial_value=np.asarray(charges, dtype=np.float64).reshape(n, 1))
    return st


def array_of(obj):
    """The array behind a dat-like object (numpy array or torch tensor)."""
    if isinstance(obj, np.ndarray) or _is_torch(obj):
        return obj
    if hasattr(obj, "data"):
        return obj.data
    return obj


def _is_torch(x):
    return type(x).__module__.startswith("torch")
