"""KMCFMM: the user-facing FMM-KMC interface, GB300 implementation.

Same constructor and methods as coulomb_kmc.KMCFMM (coulomb_kmc/kmc_fmm.py:436-1105):
``initialise``, ``propose``, ``propose_with_dats``, ``accept``, ``free`` and the
``energy`` attribute.  All arithmetic runs in libkmc_gb300.so on the current
CUDA device; PyTorch only provides device buffers and the stream.  There is no
CPU fallback.

Inputs may be ppmd-style dats (anything with ``.data``), numpy arrays, or, for
``propose_with_dats``, torch CUDA tensors (then nothing is copied between host
and device).
"""
import ctypes
from ctypes import byref, c_double, c_int64, c_void_p, POINTER
from math import ceil, log

import numpy as np

from . import _native
from .common import BCType
from .dats import array_of, _is_torch
from .lattice import lattice_operator

REAL = ctypes.c_double
INT64 = ctypes.c_int64


def _torch():
    import torch
    return torch


def _host(a, dtype):
    if _is_torch(a):
        a = a.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(a), dtype=dtype)


class KMCFMM:
    """Electrostatic energy differences for kinetic Monte Carlo (see coulomb_kmc.KMCFMM).

    :arg positions: PositionDat (n,3) float64, numpy array or tensor of charge positions.
    :arg charges: ParticleDat (n,1) float64 (or array) of charge values.
    :arg domain: object with ``extent`` (cubic box [-E/2, E/2]^3), or the edge length.
    :arg N: number of charges (optional; taken from ``positions``).
    :arg boundary_condition: 'pbc', 'free_space' or '27'.
    :arg r: number of FMM levels (finest level has 2^(r-1) cells per side).  Default
        max(2, ceil(log8(N/8))).
    :arg l: number of expansion terms (default 12).
    :arg max_move: maximum per-axis displacement of a proposed move (default: box edge).
    :arg energy_unit: multiplies all energies.
    :arg precision: 'fp64' (default, the drop-in), 'mixed' (FP32 / double-FP32 propose,
        double-FP32 accept contributions added to the FP64 state) or 'mixed_fp64_accept'.
    :arg initial_solve: 'auto' (default), 'exact' (direct particle-to-local sum) or 'fmm'
        (octree P2M/M2M/M2L/L2L, the reference's method, kmc_fmm.py:956-959); 'auto' takes
        the exact sum while cells x charges x images <= 1e8.
    ``shell_width``, ``_debug`` and ``cuda_direct`` are accepted for signature
    compatibility and have no effect (the whole path always runs on the GPU).
    """

    def __init__(self, positions, charges, domain, N=None, boundary_condition="pbc", r=None, shell_width=0.0,
                 energy_unit=1.0, _debug=False, l=None, max_move=None, cuda_direct=False, mirror_direction=None,
                 precision="fp64", initial_solve="auto"):
        self._bc = BCType(boundary_condition)
        self.boundary_condition = self._bc
        if self._bc == BCType.FF_ONLY:
            raise NotImplementedError("boundary_condition='ff-only' is not part of this implementation")
        if mirror_direction is not None:
            raise NotImplementedError("mirror charges (Dirichlet boundaries) are not part of this implementation")
        self.positions = positions
        self.charges = charges
        self.domain = domain
        self.group = getattr(positions, "group", None)
        ext = np.atleast_1d(np.asarray(getattr(domain, "extent", domain), dtype=np.float64))
        if ext.size == 1:
            ext = np.repeat(ext, 3)
        if not (abs(ext[0] - ext[1]) < 1e-14 and abs(ext[0] - ext[2]) < 1e-14):
            raise ValueError("only cubic domains are supported")
        self.extent = float(ext[0])
        pos = array_of(positions)
        n = int(pos.shape[0]) if N is None else int(N)
        self.N = n
        if r is None:
            r = max(2, int(ceil(log(max(n / 8.0, 1.0), 8)))) if n > 8 else 2
        self.R = int(r)
        self.L = int(l) if l is not None else 12
        self.energy_unit = float(energy_unit)
        self.max_move = float(max_move) if max_move is not None else float(np.max(ext))
        self.cuda_direct = cuda_direct
        self.precision = precision
        self._energy = None
        self._energy_valid = False
        self._handle = None
        self._staging = {}
        L = _native.lib()
        prm = _native.KmcParams()
        prm.boundary = _native.KMC_BC[self._bc.value]
        prm.r = self.R
        prm.l = self.L
        prm.precision = _native.KMC_PREC[precision]
        prm.extent = self.extent
        prm.max_move = self.max_move
        prm.energy_unit = self.energy_unit
        if initial_solve not in _native.KMC_INIT:
            raise ValueError("initial_solve must be one of %s" % sorted(_native.KMC_INIT))
        prm.initial_solve = _native.KMC_INIT[initial_solve]
        if self._bc == BCType.PBC:
            data, indptr, indices, dip = lattice_operator(self.L, self.extent)
            self._lr = (data, indptr, indices, dip)
            prm.lr_nnz = len(data)
            prm.lr_data = data.ctypes.data_as(POINTER(c_double))
            prm.lr_indptr = indptr.ctypes.data_as(POINTER(c_int64))
            prm.lr_indices = indices.ctypes.data_as(POINTER(c_int64))
            for i in range(3):
                prm.lr_dipole[i] = dip[i]
        h = c_void_p()
        _native.check(L.kmc_create(byref(prm), byref(h)), "kmc_create")
        self._handle = h

    # ------------------------------------------------------------------
    @property
    def energy(self):
        """Total system energy (valid after initialise)."""
        if self._handle is None or self._energy is None:
            return self._energy
        if not self._energy_valid:
            e = c_double()
            _native.check(_native.lib().kmc_get_energy(self._handle, byref(e)), "kmc_get_energy")
            self._energy = e.value
            self._energy_valid = True
        return self._energy

    def _assert_init(self):
        if self._energy is None:
            raise RuntimeError("Run initialise before this call")

    def _set_stream(self):
        torch = _torch()
        if torch.cuda.is_available():
            _native.lib().kmc_set_stream(self._handle, c_void_p(torch.cuda.current_stream().cuda_stream))

    def initialise(self):
        """Initial solve: cell store, finest-level local expansions, energy (kmc_fmm.py:947-993)."""
        pos = _host(array_of(self.positions), np.float64).reshape(-1, 3)
        q = _host(array_of(self.charges), np.float64).reshape(-1)
        if pos.shape[0] != self.N or q.shape[0] != self.N:
            raise ValueError("positions and charges must have N entries")
        self._check_in_box(pos)
        self._set_stream()
        e = c_double()
        _native.check(_native.lib().kmc_initialise(self._handle, self.N, pos.ctypes.data, q.ctypes.data, byref(e)),
                      "kmc_initialise")
        self._energy = e.value
        self._energy_valid = True
        self._charges_host = q

    def _check_in_box(self, pos):
        h = 0.5 * self.extent
        if np.any(pos < -h) or np.any(pos > h):
            raise RuntimeError("Charge position is outside simulation domain.")

    def _positions_host(self):
        return array_of(self.positions)

    def _check_move_valid(self, old_pos, new_pos):
        """kmc_mpi_decomp.py:312-345"""
        e = self.extent
        for d in range(3):
            if np.any(new_pos[:, d] < -0.5 * e) or np.any(new_pos[:, d] > 0.5 * e):
                raise RuntimeError("Proposed position is outside simulation domain. Extent {}, dimension {}, "
                                   "value {}.".format(e, d, new_pos[:, d]))
        periodic = self._bc != BCType.FREE_SPACE
        for mx in new_pos:
            rvec = mx - old_pos
            if periodic:
                for d in range(3):
                    if rvec[d] < -0.5 * e:
                        rvec[d] += e
                    if rvec[d] > 0.5 * e:
                        rvec[d] -= e
            if np.any(np.abs(rvec) > self.max_move):
                raise RuntimeError("Proposed move violates max_move. Old position {}, new position {}.".format(
                    old_pos, mx))

    # ------------------------------------------------------------------
    def propose(self, moves):
        """Total energies of proposed moves: moves = ((id, (k,3) array), ...) (kmc_fmm.py:774-787)."""
        self._assert_init()
        nump = len(moves)
        movs = [np.atleast_2d(np.asarray(m[1], dtype=np.float64)) for m in moves]
        pids = np.array([int(m[0]) for m in moves], dtype=np.int64)
        counts = np.array([m.shape[0] for m in movs], dtype=np.int64)
        es = np.zeros(nump + 1, dtype=np.int64)
        es[1:] = np.cumsum(counts)
        pos = self._positions_host()
        pos_h = _host(pos, np.float64).reshape(-1, 3)
        for pid, mv in zip(pids, movs):
            self._check_move_valid(pos_h[pid], mv)
        newp = np.ascontiguousarray(np.concatenate(movs, axis=0), dtype=np.float64)
        diffs = np.zeros(int(es[-1]), dtype=np.float64)
        self._set_stream()
        _native.check(_native.lib().kmc_propose_moves(self._handle, nump, pids.ctypes.data, es.ctypes.data,
                                                      newp.ctypes.data, diffs.ctypes.data), "kmc_propose_moves")
        energy = self.energy
        out = []
        for i, (pid, mv) in enumerate(zip(pids, movs)):
            e = np.zeros(mv.shape[0])
            for j, mx in enumerate(mv):
                if np.linalg.norm(pos_h[pid, :] - mx) < 10.0 ** -14:
                    e[j] = energy
                else:
                    e[j] = energy + diffs[es[i] + j]
            out.append(e)
        return tuple(out)

    # ------------------------------------------------------------------
    def _pinned(self, name, n, torch_dtype):
        """A persistent page-locked host array of at least n elements."""
        torch = _torch()
        buf = self._staging.get(name)
        if buf is None or buf.numel() < n:
            buf = torch.empty(max(n, 1), dtype=torch_dtype, pin_memory=True)
            self._staging[name] = buf
        return buf

    def host_buffers(self, max_prop):
        """Pinned host arrays for the host path of propose_with_dats: prop_positions
        (N, 3 max_prop), prop_masks (N, max_prop), current_sites (N, 1) and
        prop_energy_diffs (N, max_prop).  A caller that fills them in place and passes
        them saves the copies into and out of the staging buffers (the data goes
        between these pages and the device directly).  They stay valid while the
        system's size and max_prop do not change."""
        torch = _torch()
        n, M = self.N, int(max_prop)
        out = {}
        for key, name, shape, dt in (("prop_positions", "ppos", (n, 3 * M), torch.float64),
                                     ("prop_masks", "mask", (n, M), torch.int64),
                                     ("current_sites", "sites", (n, 1), torch.int64),
                                     ("prop_energy_diffs", "pde", (n, M), torch.float64)):
            h = self._pinned(name, n * shape[1], dt)
            out[key] = h[:n * shape[1]].numpy().reshape(shape)
        return out

    def release_host_buffers(self):
        """Drop the page-locked arrays host_buffers returned (the next call to it
        allocates them again)."""
        self._staging = {}

    def propose_with_dats(self, site_max_counts, current_sites, prop_positions, prop_masks, prop_energy_diffs,
                          diff=True, prop_charges=None, sync=True):
        """Energy differences of masked proposals written into prop_energy_diffs (kmc_fmm.py:665-762).

        With torch CUDA tensors for all arrays the call is device resident; ``sync=False`` then skips
        the host read of the move-validation counter (call ``check_errors()`` later).
        """
        self._assert_init()
        if not diff:
            raise NotImplementedError()
        smc, sites = array_of(site_max_counts), array_of(current_sites)
        ppos, pmask, pde = array_of(prop_positions), array_of(prop_masks), array_of(prop_energy_diffs)
        pq = array_of(prop_charges) if prop_charges is not None else None
        M = int(pmask.shape[1])
        if int(pde.shape[1]) != M or int(ppos.shape[1]) != 3 * M:
            raise AssertionError("prop_energy_diffs/prop_positions strides must match prop_masks")
        nsite = int(np.prod(smc.shape))
        L = _native.lib()
        self._set_stream()
        if all(_is_torch(a) and a.is_cuda for a in (smc, sites, ppos, pmask, pde)) and \
                (pq is None or (_is_torch(pq) and pq.is_cuda)):
            torch = _torch()
            for a, dt in ((smc, torch.int64), (sites, torch.int64), (pmask, torch.int64), (ppos, torch.float64),
                          (pde, torch.float64)):
                if a.dtype != dt or not a.is_contiguous():
                    raise TypeError("device dats must be contiguous int64/float64 tensors")
            _native.check(L.kmc_propose_with_dats(self._handle, self.N, M, nsite, smc.data_ptr(), sites.data_ptr(),
                                                  ppos.data_ptr(), pmask.data_ptr(),
                                                  pq.data_ptr() if pq is not None else None, pde.data_ptr()),
                          "kmc_propose_with_dats")
            if sync:
                self.check_errors()
            return
        # host arrays: one library call copies them to the device (page-locked ones, as
        # host_buffers gives, by DMA), evaluates and copies the differences back
        a_smc = _host(smc, np.int64)
        a_sites = _host(sites, np.int64)
        a_ppos = _host(ppos, np.float64)
        a_mask = _host(pmask, np.int64)
        a_pq = _host(pq, np.float64) if pq is not None else None
        direct = (isinstance(pde, np.ndarray) and pde.dtype == np.float64 and pde.flags.c_contiguous
                  and pde.flags.writeable)
        a_pde = pde if direct else _host(pde, np.float64).copy()
        errs = (c_int64 * 2)()
        _native.check(L.kmc_propose_with_dats_host(self._handle, self.N, M, nsite, a_smc.ctypes.data,
                                                   a_sites.ctypes.data, a_ppos.ctypes.data, a_mask.ctypes.data,
                                                   a_pq.ctypes.data if a_pq is not None else None,
                                                   a_pde.ctypes.data, errs), "kmc_propose_with_dats_host")
        if errs[1] > 0:
            raise RuntimeError("A cell store overflowed during a device-selected accept.")
        if errs[0] > 0:
            raise RuntimeError("Bad proposed move was detected.")
        if not direct:
            if _is_torch(pde):
                pde.copy_(_torch().from_numpy(a_pde.reshape(tuple(pde.shape))))
            else:
                pde[...] = a_pde.reshape(pde.shape)

    def error_counts(self):
        """(invalid proposed moves, store overflows) counted on the device since the last
        read; reading clears them (synchronises)."""
        bad, ovf = c_int64(), c_int64()
        _native.check(_native.lib().kmc_get_error(self._handle, byref(bad), byref(ovf)), "kmc_get_error")
        return bad.value, ovf.value

    def check_errors(self):
        """Raise RuntimeError if any proposed move since the last check was invalid."""
        bad, ovf = self.error_counts()
        if ovf > 0:
            raise RuntimeError("A cell store overflowed during a device-selected accept.")
        if bad > 0:
            raise RuntimeError("Bad proposed move was detected.")

    # ------------------------------------------------------------------
    def accept(self, move=None):
        """Accept move = (id, new_position): updates the energy, the GPU state and the positions dat
        (kmc_fmm.py:789-912)."""
        self._assert_init()
        if move is None:
            raise RuntimeError("No moves to accept were passed.")
        pid = int(move[0])
        newp = np.ascontiguousarray(np.asarray(move[1], dtype=np.float64).reshape(3))
        pos = self._positions_host()
        old = _host(pos[pid], np.float64).reshape(3)
        self._check_move_valid(old, newp.reshape(1, 3))
        self._set_stream()
        _native.check(_native.lib().kmc_accept(self._handle, pid, newp.ctypes.data_as(POINTER(c_double))),
                      "kmc_accept")
        self._energy_valid = False
        if _is_torch(pos):
            pos[pid, :] = _torch().from_numpy(newp).to(pos.device)
        else:
            pos[pid, :] = newp

    def accept_device(self, d_pid, d_new_position, d_energy_diff):
        """Accept a move selected on the device (int64[1], float64[3], float64[1] CUDA tensors).

        Does not synchronise and does not update a host positions dat; read the
        positions back with ``state()`` when needed."""
        self._assert_init()
        self._set_stream()
        _native.check(_native.lib().kmc_accept_device(self._handle, d_pid.data_ptr(), d_new_position.data_ptr(),
                                                      d_energy_diff.data_ptr()), "kmc_accept_device")
        self._energy_valid = False

    def autotune(self, reps=5):
        """Time the launch-shape candidates that leave every result bit-identical and keep
        the fastest (kmc_autotune); returns {key: value} of all tuning keys.  The lattice
        kernels are tuned on the proposals of the last propose, so call it after one."""
        self._assert_init()
        self._set_stream()
        out = (ctypes.c_int32 * _native.NTUNE)()
        _native.check(_native.lib().kmc_autotune(self._handle, int(reps), out), "kmc_autotune")
        return {k: int(out[k]) for k in range(_native.NTUNE)}

    def set_tuning(self, key, value):
        """Set one launch-shape tuning key (kmc_set_tuning)."""
        _native.check(_native.lib().kmc_set_tuning(self._handle, int(key), int(value)), "kmc_set_tuning")

    def get_tuning(self, key):
        """The value of one launch-shape tuning key (kmc_get_tuning; 0: the built-in choice)."""
        v = ctypes.c_int32()
        _native.check(_native.lib().kmc_get_tuning(self._handle, int(key), ctypes.byref(v)), "kmc_get_tuning")
        return int(v.value)

    def reserve_store(self, capacity):
        """Set the cell store's capacity (slots per cell) to at least ``capacity`` and the
        largest occupancy (kmc_store_reserve); returns the new capacity.  Synchronises; a
        driver captures its step again by itself."""
        self._assert_init()
        self._set_stream()
        _native.check(_native.lib().kmc_store_reserve(self._handle, int(capacity)), "kmc_store_reserve")
        return self.max_occupancy()[1]

    def max_occupancy(self):
        """(largest cell occupancy, store capacity); synchronises."""
        self._assert_init()
        mx, cap = c_int64(), c_int64()
        _native.check(_native.lib().kmc_max_occupancy(self._handle, byref(mx), byref(cap)), "kmc_max_occupancy")
        return mx.value, cap.value

    def resolve_overflow(self):
        """Apply a device-selected accept that was refused because its new cell was full,
        after growing the store (kmc_resolve_overflow); True if a move was applied."""
        self._assert_init()
        self._set_stream()
        a = c_int64()
        _native.check(_native.lib().kmc_resolve_overflow(self._handle, byref(a)), "kmc_resolve_overflow")
        self._energy_valid = False
        return bool(a.value)

    # ------------------------------------------------------------------
    def state(self):
        """Device state copied to host: positions, cells, occupancy, reference-layout local
        expansions [ncell, 2L^2] and (pbc) the level-0 multipole."""
        ncell, cap, n = c_int64(), c_int64(), c_int64()
        L = _native.lib()
        L.kmc_info(self._handle, byref(ncell), byref(cap), byref(n))
        pos = np.zeros((n.value, 3))
        cells = np.zeros(n.value, np.int64)
        occ = np.zeros(ncell.value, np.int64)
        lexp = np.zeros((ncell.value, 2 * self.L * self.L))
        mp = np.zeros(2 * self.L * self.L)
        _native.check(L.kmc_read_state(self._handle, pos.ctypes.data, cells.ctypes.data, occ.ctypes.data,
                                       lexp.ctypes.data, mp.ctypes.data), "kmc_read_state")
        return {"positions": pos, "cells": cells, "occupancy": occ, "local_expansions": lexp, "multipole": mp,
                "capacity": cap.value}

    def free(self):
        """Release the GPU state (kmc_fmm.py:569-577)."""
        if self._handle is not None:
            self._set_stream()  # the stream last bound (a driver's) may no longer exist
            _native.lib().kmc_free(self._handle)
            self._handle = None
        self._staging = {}

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    # ------------------------------------------------------------------
    # insertion and removal of charges (InjectorExtractor, kmc_inject_extract.py)
    def get_energy(self, ids):
        """Energy of groups of charges in the system: ``ids`` (n, m) local ids, returns the
        n sums of q_i phi_i (phi without the charge itself) times the energy unit
        (kmc_inject_extract.py:82-123)."""
        self._assert_init()
        torch = _torch()
        ids = np.atleast_2d(np.asarray(ids, dtype=np.int64))
        flat = np.ascontiguousarray(ids.ravel())
        if flat.size == 0:
            return np.zeros(ids.shape[0])
        if np.any(flat < 0) or np.any(flat >= self.N):
            raise IndexError("charge id out of range")
        self._set_stream()
        d_ids = torch.from_numpy(flat).cuda()
        out = torch.empty(flat.size, dtype=torch.float64, device="cuda")
        _native.check(_native.lib().kmc_get_energy_ids(self._handle, flat.size, d_ids.data_ptr(), out.data_ptr()),
                      "kmc_get_energy_ids")
        return out.cpu().numpy().reshape(ids.shape).sum(axis=1)

    def get_energy_with_dats(self, masks, energy):
        """Write get_energy of every charge with a positive mask into ``energy``
        (kmc_inject_extract.py:125-142)."""
        m = _host(array_of(masks), np.int64).reshape(self.N, -1)[:, 0]
        ids = np.nonzero(m > 0)[0]
        e = self.get_energy(ids.reshape(-1, 1))
        tgt = array_of(energy)
        if _is_torch(tgt):
            tgt[ids, 0] = _torch().from_numpy(e).to(tgt.device, tgt.dtype)
        else:
            tgt[ids, 0] = e

    def compute_energy(self, positions, charges):
        """Energy of a small set of charges alone in the box (the reference's direct
        solvers, kmc_inject_extract.py:145-166), times the energy unit."""
        torch = _torch()
        pos = np.ascontiguousarray(np.atleast_2d(_host(positions, np.float64)).reshape(-1, 3))
        q = np.ascontiguousarray(_host(charges, np.float64).reshape(-1))
        if q.shape[0] != pos.shape[0]:
            raise ValueError("positions and charges differ in length")
        self._set_stream()
        dp, dq = torch.from_numpy(pos).cuda(), torch.from_numpy(q).cuda()
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        _native.check(_native.lib().kmc_group_energy(self._handle, q.shape[0], dp.data_ptr(), dq.data_ptr(),
                                                      out.data_ptr()), "kmc_group_energy")
        return float(out.item())

    def propose_extract(self, ids, self_energy=True):
        """Energy change of removing each group of charges (rows of ``ids``)
        (kmc_inject_extract.py:178-214)."""
        self._assert_init()
        ids = np.atleast_2d(np.asarray(ids, dtype=np.int64))
        if ids.size == 0:
            return np.array(())
        group = self.get_energy(ids)
        pos = self._positions_now()
        q = self._charges_now()
        out = np.zeros(ids.shape[0])
        for g in range(ids.shape[0]):
            bb = self.compute_energy(pos[ids[g]], q[ids[g]]) if self_energy else 0.0
            out[g] = bb - group[g]
        return out

    def propose_inject(self, positions, charges):
        """Energy change of adding the charges (kmc_inject_extract.py:217-237)."""
        self._assert_init()
        pos = np.atleast_2d(_host(positions, np.float64)).reshape(-1, 3)
        q = _host(charges, np.float64).reshape(-1)
        bb = self.compute_energy(pos, q)
        phi = self.eval_field(pos)
        return bb + self.energy_unit * float(np.sum(q * phi))

    def extract(self, ids=()):
        """Remove the charges ``ids`` (kmc_inject_extract.py:240-301); the others keep
        their order and the positions / charges dats are shortened accordingly."""
        self._assert_init()
        ids = np.ascontiguousarray(np.asarray(ids, dtype=np.int64).ravel())
        if ids.size == 0:
            return
        self._set_stream()
        de = c_double()
        _native.check(_native.lib().kmc_extract(self._handle, ids.size, ids.ctypes.data, byref(de)), "kmc_extract")
        keep = np.setdiff1d(np.arange(self.N), ids)
        self._replace_rows(keep, None, None)
        self._energy_valid = False

    def inject(self, add):
        """Add charges, appended after the existing ones (kmc_inject_extract.py:304-424).
        ``add`` maps the positions and charges dats to the new rows (as the reference's
        ``state.modifier.add``) or is a (positions, charges) pair."""
        self._assert_init()
        if isinstance(add, dict):
            pos, q = add[self.positions], add[self.charges]
        else:
            pos, q = add
        pos = np.ascontiguousarray(np.atleast_2d(_host(pos, np.float64)).reshape(-1, 3))
        q = np.ascontiguousarray(_host(q, np.float64).reshape(-1))
        if q.shape[0] != pos.shape[0] or q.shape[0] == 0:
            raise ValueError("inject needs as many charges as positions")
        self._check_in_box(pos)
        self._set_stream()
        de = c_double()
        _native.check(_native.lib().kmc_inject(self._handle, q.shape[0], pos.ctypes.data, q.ctypes.data, byref(de)),
                      "kmc_inject")
        self._replace_rows(np.arange(self.N), pos, q)
        self._energy_valid = False

    def _positions_now(self):
        return self.state()["positions"]

    def _charges_now(self):
        return _host(array_of(self.charges), np.float64).reshape(self.N, -1)[:, 0]

    def _replace_rows(self, keep, add_pos, add_q):
        """Host dats after extract (rows ``keep``) or inject (rows appended)."""
        pos = self.state()["positions"]
        q = self._charges_now()[keep]
        if add_q is not None:
            q = np.concatenate([q, add_q])
        self.N = pos.shape[0]
        for attr, new in (("positions", pos), ("charges", q.reshape(-1, 1))):
            obj = getattr(self, attr)
            if hasattr(obj, "data") and isinstance(getattr(obj, "data"), np.ndarray):
                obj.data = new.copy()
            elif _is_torch(obj):
                setattr(self, attr, _torch().from_numpy(new.copy()).to(obj.device))
            else:
                setattr(self, attr, new.copy())
        self._charges_host = q.copy()

    def eval_field(self, points):
        """Potential of all charges at the given (n, 3) points (kmc_fmm.py:544-567); the
        energy unit is not applied.  numpy in, numpy out; a CUDA tensor in, a CUDA tensor
        out (no host copy)."""
        self._assert_init()
        torch = _torch()
        self._set_stream()
        if _is_torch(points) and points.is_cuda:
            pts = points.detach().to(torch.float64).reshape(-1, 3).contiguous()
            out = torch.empty(pts.shape[0], dtype=torch.float64, device=pts.device)
            _native.check(_native.lib().kmc_eval_field(self._handle, pts.shape[0], pts.data_ptr(), out.data_ptr()),
                          "kmc_eval_field")
            return out
        pts = np.atleast_2d(_host(points, np.float64)).reshape(-1, 3)
        self._check_in_box(pts)
        d = torch.from_numpy(pts).cuda()
        out = torch.empty(pts.shape[0], dtype=torch.float64, device="cuda")
        _native.check(_native.lib().kmc_eval_field(self._handle, pts.shape[0], d.data_ptr(), out.data_ptr()),
                      "kmc_eval_field")
        return out.cpu().numpy()
