"""CPU oracle for the FMM-KMC energy-difference path (TEST INFRASTRUCTURE ONLY).

Restates ppmd/coulomb_kmc's single-rank propose/accept path on the CPU, in the
reference's own data layout (halo-padded particle store and local-expansion
store, reference component order), driving the C restatement in
``kmc_oracle.c``.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may use it; the GPU product never imports it.

Deliberate, documented departures from the reference (the reference cannot run
here because ppmd is absent):

* The initial finest-level local expansions are the exact particle-to-local
  sums of every well-separated charge image (``orc_init_local_exp``), i.e. the
  state the reference's ``accept_local_exp`` maintains incrementally, instead
  of ppmd PyFMM's tree solve.  The initial energy is assembled from the same
  near-field and expansion terms (``0.5 * sum_i (U0D_i + U0I_i)`` plus the
  lattice term for pbc).
* The lattice operator for pbc (ppmd ``LongRangeMTL``) is an input: callers
  pass the CSR operator and dipole coefficients.
* Cell binning everywhere uses the C ``get_cell`` rule
  (kmc_mpi_decomp.py:400-420), also for accepted moves.
"""
import ctypes
import os
import subprocess
from ctypes import c_double, c_int64, POINTER

import numpy as np

REAL = np.float64
INT64 = np.int64

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libkmc_oracle.so")
_lib = None

# common.py:53-81
CELL_OFFSETS = np.array([(x, y, z) for z in (-1, 0, 1) for y in (-1, 0, 1) for x in (-1, 0, 1)], dtype=INT64)


def build():
    """Compile the oracle shared library with its Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _lib.orc_local_eval.restype = c_double
        _lib.orc_lr_energy.restype = c_double
        _lib.orc_direct_energy.restype = c_double
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def spherical(xyz):
    """common.py:6-34"""
    x, y, z = xyz
    xy = x * x + y * y
    return np.array((np.sqrt(xy + z * z), np.arctan2(np.sqrt(xy), z), np.arctan2(y, x)))


def multipole_exp(L, sph, charge, out):
    lib().orc_multipole_exp(c_int64(L), c_double(charge), c_double(sph[0]), c_double(sph[1]), c_double(sph[2]), _p(out))


def dot_vec(L, sph, charge, out):
    lib().orc_dot_vec(c_int64(L), c_double(charge), c_double(sph[0]), c_double(sph[1]), c_double(sph[2]), _p(out))


def local_exp(L, sph, charge, out):
    lib().orc_local_exp(c_int64(L), c_double(charge), c_double(sph[0]), c_double(sph[1]), c_double(sph[2]), _p(out))


def local_eval(L, sph, moments):
    m = np.ascontiguousarray(moments, dtype=REAL)
    return lib().orc_local_eval(c_int64(L), c_double(sph[0]), c_double(sph[1]), c_double(sph[2]), _p(m))


def direct_energy(bc, E, positions, charges):
    """FreeSpaceDirect / NearestDirect restated (tests/host/test_common.py:24-103)."""
    P = np.ascontiguousarray(positions, dtype=REAL)
    Q = np.ascontiguousarray(np.ravel(charges), dtype=REAL)
    return lib().orc_direct_energy(c_int64(0 if bc == "free_space" else 1), c_double(E), c_int64(len(Q)), _p(P), _p(Q))


class OracleKMC:
    """Reference-layout CPU restatement of ``KMCFMM`` (single rank).

    Mirrors ``KMCFMM.initialise/propose/propose_with_dats/accept``
    (coulomb_kmc/kmc_fmm.py:436-1105) and the components it wires together.
    ``positions`` (N,3) and ``charges`` (N,) are numpy arrays owned by the
    caller; ``accept`` updates ``positions`` in place like the reference does.
    """

    def __init__(self, positions, charges, extent, r, l, boundary_condition="pbc", max_move=None,
                 energy_unit=1.0, lr_operator=None):
        lib()
        self.positions = positions
        self.charges = np.ascontiguousarray(np.ravel(charges), dtype=REAL)
        self.N = positions.shape[0]
        self.E = float(extent)
        self.extent = np.array([self.E] * 3, dtype=REAL)
        self.R = int(r)
        self.L = int(l)
        self.bc = boundary_condition
        assert self.bc in ("free_space", "27", "pbc")
        self.periodic = 0 if self.bc == "free_space" else 1
        self.energy_unit = float(energy_unit)
        self.max_move = float(max_move) if max_move is not None else self.E
        self.ncps = 2 ** (self.R - 1)
        cw = self.E / self.ncps
        # kmc_mpi_decomp.py:72
        self.pad = 2 + int(np.ceil(self.max_move / cw))
        self.lsd = self.ncps + 2 * self.pad
        offs = np.arange(-self.pad, self.ncps + self.pad)
        self.cell_indices = offs % self.ncps  # wrapped primary index per store index
        self.periodic_factors = offs // self.ncps
        self.cell_offsets = offs
        lsd = self.lsd
        # 27 neighbour offsets as linear store offsets: kmc_local.py:137-139
        self.offsets_arr = np.array([ox[0] + lsd * (ox[1] + lsd * ox[2]) for ox in CELL_OFFSETS], dtype=INT64)
        self.ids = np.arange(self.N, dtype=INT64)
        self.energy = None
        if self.bc == "pbc":
            assert lr_operator is not None, "pbc needs the lattice operator"
            d, ip, ix, dip = lr_operator
            self.lr_data = np.ascontiguousarray(d, dtype=REAL)
            self.lr_indptr = np.ascontiguousarray(ip, dtype=INT64)
            self.lr_indices = np.ascontiguousarray(ix, dtype=INT64)
            self.lr_dip = np.ascontiguousarray(dip, dtype=REAL)
        self._compute_centres()

    # ------------------------------------------------------------------
    def _compute_centres(self):
        """kmc_octal.py:397-428"""
        lsd, E, w = self.lsd, self.E, self.E / self.ncps
        start = -0.5 * E + 0.5 * w
        c1 = start + self.cell_offsets * w
        c0 = start + self.cell_indices * w
        self.cell_centres = np.zeros((lsd, lsd, lsd, 3), dtype=REAL)
        self.orig_cell_centres = np.zeros_like(self.cell_centres)
        self.cell_centres[..., 0] = c1[None, None, :]
        self.cell_centres[..., 1] = c1[None, :, None]
        self.cell_centres[..., 2] = c1[:, None, None]
        self.orig_cell_centres[..., 0] = c0[None, None, :]
        self.orig_cell_centres[..., 1] = c0[None, :, None]
        self.orig_cell_centres[..., 2] = c0[:, None, None]

    def _bin(self, pos):
        pos = np.ascontiguousarray(np.atleast_2d(pos), dtype=REAL)
        out = np.zeros(pos.shape[0], dtype=INT64)
        lib().orc_bin_cells(c_int64(pos.shape[0]), _p(pos), _p(self.extent), c_int64(self.ncps), _p(out))
        return out

    def _tuple(self, c):
        n = self.ncps
        return (int(c % n), int((c // n) % n), int(c // (n * n)))

    def lcell(self, c):
        x, y, z = self._tuple(c)
        p, lsd = self.pad, self.lsd
        return (x + p) + lsd * ((y + p) + lsd * (z + p))

    # ------------------------------------------------------------------
    def initialise(self, local_expansions=None):
        """KMCFMM.initialise (kmc_fmm.py:947-993) with the exact P2L initial solve.

        ``local_expansions`` optionally supplies the primary-cell expansions
        ([ncps^3, 2L^2], reference layout) instead of computing them.
        """
        N, L, lsd = self.N, self.L, self.lsd
        self.fmm_cells = self._bin(self.positions)
        self._build_store()
        NC = 2 * L * L
        ncell = self.ncps ** 3
        if local_expansions is None:
            prim = np.zeros((ncell, NC), dtype=REAL)
            pos = np.ascontiguousarray(self.positions, dtype=REAL)
            lib().orc_init_local_exp(c_int64(L), c_int64(self.periodic), _p(self.extent), c_int64(self.ncps),
                                     c_int64(N), _p(pos), _p(self.charges), _p(self.fmm_cells), _p(prim))
        else:
            prim = np.ascontiguousarray(local_expansions, dtype=REAL).reshape(ncell, NC)
        ci = self.cell_indices
        lin = ci[None, None, :] + self.ncps * (ci[None, :, None] + self.ncps * ci[:, None, None])
        self.local_expansions = np.ascontiguousarray(prim[lin.ravel()].reshape(lsd, lsd, lsd, NC))
        # initial energy from the same near/far terms as propose: 0.5 sum_i (U0D + U0I)
        h = self._setup_all_particles()
        u0d = np.zeros(N, REAL)
        u0i = np.zeros(N, REAL)
        self._direct(1, N, h["old_positions"], h["old_charges"], h["old_ids"], h["old_fmm_cells"], u0d)
        self._indirect(N, h["old_fmm_cells"], h["old_positions"], h["old_charges"], u0i)
        energy = 0.5 * (np.sum(u0d) + np.sum(u0i))
        if self.bc == "pbc":
            # kmc_full_long_range.py:83-118
            self.multipole_exp = np.zeros(NC, REAL)
            self.local_dot_coeffs = np.zeros(NC, REAL)
            for px in range(N):
                sph = spherical(self.positions[px, :])
                multipole_exp(L, sph, self.charges[px], self.multipole_exp)
                dot_vec(L, sph, self.charges[px], self.local_dot_coeffs)
            energy += self._lr_old_energy()
        self.energy = energy * self.energy_unit
        return self.energy

    def _lr_energy_of(self, M, E):
        M = np.ascontiguousarray(M, dtype=REAL)
        E = np.ascontiguousarray(E, dtype=REAL)
        return lib().orc_lr_energy(c_int64(self.L), _p(self.lr_data), _p(self.lr_indptr), _p(self.lr_indices),
                                   _p(self.lr_dip), _p(M), _p(E))

    def _lr_old_energy(self):
        return lib().orc_lr_energy(c_int64(self.L), _p(self.lr_data), _p(self.lr_indptr), _p(self.lr_indices),
                                   _p(self.lr_dip), _p(self.multipole_exp), _p(self.local_dot_coeffs))

    def _build_store(self):
        """LocalParticleData.initialise single-rank restatement (kmc_local.py:582-825)."""
        lsd, n = self.lsd, self.ncps
        cells = self.fmm_cells
        counts = np.bincount(cells, minlength=n ** 3)
        max_occ = max(1, int(counts.max()))
        self.max_occ = max_occ
        prim = np.zeros((n ** 3, max_occ, 5), dtype=REAL)
        prim_ids = np.zeros((n ** 3, max_occ), dtype=INT64)
        fill = np.zeros(n ** 3, dtype=INT64)
        for pid in range(self.N):  # particles appended in index order
            c = cells[pid]
            k = fill[c]
            prim[c, k, 0:3] = self.positions[pid]
            prim[c, k, 3] = self.charges[pid]
            prim[c, k, 4:5].view(INT64)[0] = self.ids[pid]
            prim_ids[c, k] = self.ids[pid]
            fill[c] += 1
        ci = self.cell_indices
        lin = ci[None, None, :] + n * (ci[None, :, None] + n * ci[:, None, None])
        self.store = np.ascontiguousarray(prim[lin.ravel()].reshape(lsd, lsd, lsd, max_occ, 5))
        self.store_ids = np.ascontiguousarray(prim_ids[lin.ravel()].reshape(lsd, lsd, lsd, max_occ))
        self.occ = np.ascontiguousarray(counts[lin.ravel()].reshape(lsd, lsd, lsd)).astype(INT64)
        pf = self.periodic_factors
        for d in range(3):
            xyz = 2 - d
            shape = [1, 1, 1]
            shape[d] = lsd
            shift = (pf * self.E).reshape(shape)
            self.store[..., xyz] += shift[..., None]
        bad = np.zeros((lsd, lsd, lsd), dtype=bool)
        for d in range(3):
            shape = [1, 1, 1]
            shape[d] = lsd
            p = pf.reshape(shape)
            if self.bc == "free_space":
                bad |= np.broadcast_to(p != 0, bad.shape)
            elif self.bc == "27":
                bad |= np.broadcast_to(np.abs(p) > 1, bad.shape)
        self.occ[bad] = 0
        self.store[bad] = np.nan

    def _setup_all_particles(self):
        N = self.N
        h = {
            "old_positions": np.ascontiguousarray(self.positions, dtype=REAL).copy(),
            "old_charges": self.charges.copy(),
            "old_ids": self.ids.copy(),
            "old_fmm_cells": np.array([self.lcell(c) for c in self.fmm_cells], dtype=INT64),
        }
        return h

    # ------------------------------------------------------------------
    def _direct(self, exclude, n, pos, q, ids, cells, out):
        lib().orc_direct(c_int64(exclude), c_int64(n), _p(self.offsets_arr), _p(pos), _p(q), _p(ids), _p(cells),
                         _p(self.store), _p(self.store_ids), _p(self.occ), c_int64(self.max_occ), _p(out))

    def _indirect(self, n, cells, pos, q, out):
        lib().orc_indirect(c_int64(self.L), c_int64(n), _p(cells), _p(self.cell_centres), _p(pos), _p(q),
                           _p(self.local_expansions), _p(out))

    def _components(self, total, nump, h, stride):
        """kmcl.propose + kmco.propose + _si.propose + _lr_energy.propose"""
        u1d = np.zeros(total, REAL)
        u0d = np.zeros(nump, REAL)
        u1i = np.zeros(total, REAL)
        u0i = np.zeros(nump, REAL)
        self._direct(0, total, h["new_shifted_positions"], h["new_charges"], h["new_ids"], h["new_fmm_cells"], u1d)
        self._direct(1, nump, h["old_positions"], h["old_charges"], h["old_ids"], h["old_fmm_cells"], u0d)
        self._indirect(nump, h["old_fmm_cells"], h["old_positions"], h["old_charges"], u0i)
        self._indirect(total, h["new_fmm_cells"], h["new_shifted_positions"], h["new_charges"], u1i)
        usi = np.zeros((max(nump, 1), stride), REAL)
        lib().orc_self_interaction(c_int64(self.periodic), _p(self.extent), c_int64(stride), c_int64(nump),
                                   _p(h["exclusive_sum"]), _p(h["old_positions"]), _p(h["old_charges"]),
                                   _p(h["new_positions"]), _p(usi))
        if self.bc == "pbc":
            old_energy = self._lr_old_energy()
            lib().orc_long_range_energy(c_int64(self.L), c_double(old_energy), c_int64(stride), c_int64(nump),
                                        _p(h["exclusive_sum"]), _p(h["old_positions"]), _p(h["old_charges"]),
                                        _p(h["new_positions"]), _p(h["new_charges"]), _p(self.multipole_exp),
                                        _p(self.local_dot_coeffs), _p(self.lr_data), _p(self.lr_indptr),
                                        _p(self.lr_indices), _p(self.lr_dip), _p(usi))
        return u0d, u1d, u0i, u1i, usi

    def propose_with_dats(self, site_max_counts, current_sites, prop_positions, prop_masks, prop_energy_diffs,
                          diff=True, prop_charges=None):
        """KMCFMM.propose_with_dats (kmc_fmm.py:665-762)."""
        if self.energy is None:
            raise RuntimeError("Run initialise before this call")
        if not diff:
            raise NotImplementedError()
        N = self.N
        M = prop_masks.shape[1]
        assert prop_energy_diffs.shape[1] == M and prop_positions.shape[1] == 3 * M
        cap = (N + 1) * M
        h = {k: np.zeros(cap * w, dt) for k, w, dt in (
            ("rate_location", 1, INT64), ("new_positions", 3, REAL), ("new_charges", 1, REAL), ("new_ids", 1, INT64),
            ("new_fmm_cells", 1, INT64), ("new_shifted_positions", 3, REAL), ("old_positions", 3, REAL),
            ("old_charges", 1, REAL), ("old_ids", 1, INT64), ("old_fmm_cells", 1, INT64),
            ("exclusive_sum", 1, INT64))}
        nump = c_int64(0)
        total = c_int64(0)
        smc = np.ascontiguousarray(np.ravel(site_max_counts), dtype=INT64)
        sites = np.ascontiguousarray(np.ravel(current_sites), dtype=INT64)
        ppos = np.ascontiguousarray(prop_positions, dtype=REAL)
        pmask = np.ascontiguousarray(prop_masks, dtype=INT64)
        pq = np.ascontiguousarray(prop_charges, dtype=REAL) if prop_charges is not None else np.zeros(1, REAL)
        pos = np.ascontiguousarray(self.positions, dtype=REAL)
        err = lib().orc_setup_move(
            c_int64(N), c_int64(M), _p(smc), _p(sites), _p(pos), _p(self.charges), _p(self.ids),
            _p(self.fmm_cells), _p(ppos), _p(pmask), c_int64(1 if prop_charges is not None else 0), _p(pq),
            _p(h["rate_location"]), _p(h["new_positions"]), _p(h["new_charges"]), _p(h["new_ids"]),
            _p(h["new_fmm_cells"]), _p(h["new_shifted_positions"]), _p(h["old_positions"]), _p(h["old_charges"]),
            _p(h["old_ids"]), _p(h["old_fmm_cells"]), _p(h["exclusive_sum"]), ctypes.byref(nump),
            ctypes.byref(total), _p(self.extent), c_int64(self.ncps), c_int64(self.pad), c_int64(self.lsd),
            c_int64(self.periodic), c_double(self.max_move))
        if err > 0:
            raise RuntimeError("Bad proposed move was detected.")
        nump, total = nump.value, total.value
        if nump == 0:
            return
        stride = int(np.max(smc))
        u0d, u1d, u0i, u1i, usi = self._components(total, nump, h, stride)
        out = np.zeros(N * M, REAL)
        out[:] = np.ravel(prop_energy_diffs)
        lib().orc_diff(c_double(self.energy_unit), c_int64(nump), c_int64(stride), _p(h["exclusive_sum"]),
                       _p(h["rate_location"]), _p(u0d), _p(u0i), _p(u1d), _p(u1i), _p(usi), _p(out))
        prop_energy_diffs[...] = out.reshape(prop_energy_diffs.shape)
        self.last = dict(u0d=u0d, u1d=u1d, u0i=u0i, u1i=u1i, usi=usi, h=h, total=total, nump=nump)

    def _check_move_valid(self, old_pos, new_pos):
        """kmc_mpi_decomp.py:312-345"""
        e = self.extent
        for d in range(3):
            if np.any(new_pos[:, d] < -0.5 * e[d]) or np.any(new_pos[:, d] > 0.5 * e[d]):
                raise RuntimeError("Proposed position is outside simulation domain.")
        for mx in new_pos:
            rvec = mx - old_pos
            if self.periodic:
                for d in range(3):
                    if rvec[d] < -0.5 * e[d]:
                        rvec[d] += e[d]
                    if rvec[d] > 0.5 * e[d]:
                        rvec[d] -= e[d]
            if np.any(np.abs(rvec) > self.max_move):
                raise RuntimeError("Proposed move violates max_move.")

    def propose(self, moves):
        """KMCFMM.propose / _propose (kmc_fmm.py:774-787, 1001-1105)."""
        if self.energy is None:
            raise RuntimeError("Run initialise before this call")
        nump = len(moves)
        movs_list = [np.atleast_2d(np.asarray(m[1], dtype=REAL)) for m in moves]
        total = sum(m.shape[0] for m in movs_list)
        stride = max(m.shape[0] for m in movs_list)
        h = {"new_positions": np.zeros((total, 3), REAL), "new_charges": np.zeros(total, REAL),
             "new_ids": np.zeros(total, INT64), "new_fmm_cells": np.zeros(total, INT64),
             "old_positions": np.zeros((nump, 3), REAL), "old_charges": np.zeros(nump, REAL),
             "old_ids": np.zeros(nump, INT64), "old_fmm_cells": np.zeros(nump, INT64),
             "exclusive_sum": np.zeros(nump + 1, INT64)}
        t = 0
        for i, (mv, movs) in enumerate(zip(moves, movs_list)):
            pid = mv[0]
            self._check_move_valid(self.positions[pid], movs)
            k = movs.shape[0]
            h["old_positions"][i] = self.positions[pid]
            h["old_charges"][i] = self.charges[pid]
            h["old_ids"][i] = self.ids[pid]
            h["old_fmm_cells"][i] = self.lcell(self.fmm_cells[pid])
            h["new_positions"][t:t + k] = movs
            h["new_charges"][t:t + k] = self.charges[pid]
            h["new_ids"][t:t + k] = self.ids[pid]
            h["new_fmm_cells"][t:t + k] = [self.lcell(c) for c in self._bin(movs)]
            h["exclusive_sum"][i] = t
            t += k
        h["exclusive_sum"][nump] = t
        h["new_shifted_positions"] = h["new_positions"]
        u0d, u1d, u0i, u1i, usi = self._components(total, nump, h, stride)
        out = []
        t = 0
        for i, (mv, movs) in enumerate(zip(moves, movs_list)):
            pid = mv[0]
            e = np.zeros(movs.shape[0])
            for j, mx in enumerate(movs):
                # kmc_fmm.py:1066-1073 (operation order kept)
                udiff = +u1i[t + j] - u0d[i] + u1d[t + j] - usi[i, j] - u0i[i]
                if np.linalg.norm(self.positions[pid, :] - mx) < 10.0 ** -14:
                    e[j] = self.energy
                else:
                    e[j] = self.energy + udiff * self.energy_unit
            t += movs.shape[0]
            out.append(e)
        return tuple(out)

    # ------------------------------------------------------------------
    def _locs(self, cell_tuple_xyz):
        s2f = tuple(reversed(cell_tuple_xyz))
        locs = []
        for d in range(3):
            sel = self.cell_indices == s2f[d]
            if self.bc == "free_space":
                sel &= self.periodic_factors == 0
            elif self.bc == "27":
                sel &= np.abs(self.periodic_factors) < 2
            locs.append(np.nonzero(sel)[0].astype(INT64))
        return locs

    def accept(self, move):
        """KMCFMM._accept (kmc_fmm.py:811-912), single rank."""
        pid = int(move[0])
        new_pos = np.array(move[1], dtype=REAL).reshape(3)
        old_pos = np.array(self.positions[pid], dtype=REAL)
        charge = float(self.charges[pid])
        gid = int(self.ids[pid])
        old_cell = int(self.fmm_cells[pid])
        new_cell = int(self._bin(new_pos)[0])
        self.energy = self.propose(((pid, new_pos),))[0][0]
        self.fmm_cells[pid] = new_cell
        self.positions[pid, :] = new_pos
        # kmcl.accept: extract + inject  kmc_local.py:180-371
        lo = self._locs(self._tuple(old_cell))
        rc = lib().orc_store_extract(c_int64(gid), c_int64(len(lo[0])), _p(lo[0]), c_int64(len(lo[1])), _p(lo[1]),
                                     c_int64(len(lo[2])), _p(lo[2]), c_int64(self.lsd), c_int64(self.max_occ),
                                     _p(self.store), _p(self.store_ids), _p(self.occ))
        if rc != 0:
            raise RuntimeError("Index was not unique, this is an error.")
        ln = self._locs(self._tuple(new_cell))
        pf = [self.periodic_factors[ln[d]].astype(REAL) for d in range(3)]
        while True:
            rc = lib().orc_store_inject(c_int64(gid), _p(new_pos), c_double(charge), c_int64(len(ln[0])), _p(ln[0]),
                                        c_int64(len(ln[1])), _p(ln[1]), c_int64(len(ln[2])), _p(ln[2]), _p(pf[0]),
                                        _p(pf[1]), _p(pf[2]), c_int64(self.lsd), c_int64(self.max_occ),
                                        _p(self.extent), c_int64(self.periodic), _p(self.store),
                                        _p(self.store_ids), _p(self.occ))
            if rc != -2:
                break
            self._resize_store(self.max_occ + 1)
        # kmco.accept: accept_local_exp  kmc_octal.py:129-183
        nt = np.array(self._tuple(new_cell), dtype=INT64)
        ot = np.array(self._tuple(old_cell), dtype=INT64)
        ci = np.ascontiguousarray(self.cell_indices, dtype=INT64)
        lib().orc_accept_local_exp(c_int64(self.L), c_int64(self.periodic), _p(self.extent), c_int64(self.ncps),
                                   c_double(charge), _p(new_pos), _p(old_pos), _p(nt), _p(ot), _p(ci), _p(ci),
                                   _p(ci), c_int64(self.lsd), c_int64(self.lsd), c_int64(self.lsd),
                                   _p(self.orig_cell_centres), _p(self.local_expansions))
        if self.bc == "pbc":
            # kmc_full_long_range.py:270-316
            so, sn = spherical(old_pos), spherical(new_pos)
            multipole_exp(self.L, so, -charge, self.multipole_exp)
            dot_vec(self.L, so, -charge, self.local_dot_coeffs)
            multipole_exp(self.L, sn, charge, self.multipole_exp)
            dot_vec(self.L, sn, charge, self.local_dot_coeffs)

    def _resize_store(self, max_occ):
        """kmc_local.py:555-579"""
        lsd, old = self.lsd, self.max_occ
        st = np.zeros((lsd, lsd, lsd, max_occ, 5), REAL)
        si = np.zeros((lsd, lsd, lsd, max_occ), INT64)
        st[:, :, :, :old, :] = self.store
        si[:, :, :, :old] = self.store_ids
        self.store, self.store_ids, self.max_occ = st, si, max_occ

    # ------------------------------------------------------------------
    def eval_field(self, points):
        """KMCFMM.eval_field (kmc_fmm.py:544-567): near field (kmc_local.py:1033-1182),
        cell local expansion (kmc_octal.py:1417-1440) and, for pbc, the lattice term as
        the bilinear part of the lattice energy, E(M + m_x) - E(M) - E(m_x)
        (kmc_full_long_range.py:341-390)."""
        pts = np.ascontiguousarray(np.atleast_2d(points), dtype=REAL)
        n = pts.shape[0]
        ones = np.ones(n, REAL)
        ids = np.full(n, -1, INT64)
        cells = np.array([self.lcell(c) for c in self._bin(pts)], dtype=INT64)
        near = np.zeros(n, REAL)
        far = np.zeros(n, REAL)
        self._direct(0, n, pts, ones, ids, cells, near)
        self._indirect(n, cells, pts, ones, far)
        out = near + far
        if self.bc == "pbc":
            out += self._lr_potential(pts)
        return out

    def _lr_potential(self, pts):
        """Lattice part of the potential: bilinear part of the lattice energy for a unit charge."""
        NC = 2 * self.L * self.L
        e0 = self._lr_old_energy()
        out = np.zeros(len(pts))
        for i in range(len(pts)):
            mx = np.zeros(NC, REAL)
            ex = np.zeros(NC, REAL)
            sph = spherical(tuple(pts[i]))
            multipole_exp(self.L, sph, 1.0, mx)
            dot_vec(self.L, sph, 1.0, ex)
            out[i] = (self._lr_energy_of(self.multipole_exp + mx, self.local_dot_coeffs + ex) - e0 -
                      self._lr_energy_of(mx, ex))
        return out

    def get_energy(self, ids):
        """InjectorExtractor.get_energy (kmc_inject_extract.py:82-123): per group the sum
        of U0D + U0I + U0L of its charges (kmcl / kmco / lr get_old_energy)."""
        ids = np.atleast_2d(np.asarray(ids, dtype=INT64))
        flat = ids.ravel()
        n = flat.size
        pos = np.ascontiguousarray(self.positions[flat], dtype=REAL)
        q = np.ascontiguousarray(self.charges[flat], dtype=REAL)
        gid = np.ascontiguousarray(self.ids[flat], dtype=INT64)
        cells = np.array([self.lcell(self.fmm_cells[i]) for i in flat], dtype=INT64)
        d = np.zeros(n, REAL)
        f = np.zeros(n, REAL)
        self._direct(1, n, pos, q, gid, cells, d)
        self._indirect(n, cells, pos, q, f)
        e = d + f
        if self.bc == "pbc":
            e += q * self._lr_potential(pos)
        return (e * self.energy_unit).reshape(ids.shape).sum(axis=1)

    def compute_energy(self, positions, charges):
        """Energy of a set of charges alone in the box: pairs (3x3x3 image block for '27'
        and pbc, with self images), plus for pbc the lattice energy of the set's
        multipole (this oracle's definition of the reference's direct solvers)."""
        P = np.atleast_2d(np.asarray(positions, dtype=REAL))
        Q = np.asarray(charges, dtype=REAL).ravel()
        e = 0.0
        n = len(Q)
        shifts = [np.zeros(3)] if self.bc == "free_space" else [
            np.array([a, b, c]) * self.extent for c in (-1, 0, 1) for b in (-1, 0, 1) for a in (-1, 0, 1)]
        for i in range(n):
            for j in range(n):
                for sft in shifts:
                    if i == j and not np.any(sft):
                        continue
                    e += 0.5 * Q[i] * Q[j] / np.linalg.norm(P[i] - P[j] + sft)
        if self.bc == "pbc":
            NC = 2 * self.L * self.L
            M = np.zeros(NC, REAL)
            Ev = np.zeros(NC, REAL)
            for i in range(n):
                sph = spherical(tuple(P[i]))
                multipole_exp(self.L, sph, Q[i], M)
                dot_vec(self.L, sph, Q[i], Ev)
            e += self._lr_energy_of(M, Ev)
        return e * self.energy_unit

    def propose_extract(self, ids, self_energy=True):
        """InjectorExtractor.propose_extract (kmc_inject_extract.py:178-214)."""
        ids = np.atleast_2d(np.asarray(ids, dtype=INT64))
        g = self.get_energy(ids)
        return np.array([(self.compute_energy(self.positions[r], self.charges[r]) if self_energy else 0.0) - g[k]
                         for k, r in enumerate(ids)])

    def propose_inject(self, positions, charges):
        """InjectorExtractor.propose_inject (kmc_inject_extract.py:217-237)."""
        P = np.atleast_2d(np.asarray(positions, dtype=REAL))
        Q = np.asarray(charges, dtype=REAL).ravel()
        return self.compute_energy(P, Q) + self.energy_unit * float(np.sum(Q * self.eval_field(P)))

    def primary_local_expansions(self):
        """Primary-cell expansions in reference layout [ncps^3, 2L^2] (x fastest)."""
        n, p = self.ncps, self.pad
        return self.local_expansions[p:p + n, p:p + n, p:p + n].reshape(n ** 3, -1).copy()

    def cell_occupancy(self):
        """Primary-cell occupancy [ncps^3] (x fastest)."""
        n, p = self.ncps, self.pad
        return self.occ[p:p + n, p:p + n, p:p + n].reshape(-1).copy()
