"""The allocation-free entry point kmc_propose_moves_noalloc.

Callers that cannot allocate device memory at the moment they need energy
differences -- code running while another component owns the CUDA allocator,
or code issued inside a stream capture where a cudaMalloc would break the
capture -- use this entry point: its scratch is a fixed device array in the
library, and the caller passes only inputs and outputs (device memory).

The test calls it through the C ABI twice in a row with different moves and
checks each result against the allocating entry point kmc_propose_moves at the
1e-10 tolerance used by the other parity tests.  It is kept in its own file so
that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from conftest import neutral_charges, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _moves(rng, N, E, nump, max_k):
    pids = rng.choice(N, size=nump, replace=False).astype(np.int64)
    counts = rng.integers(1, max_k + 1, size=nump)
    es = np.zeros(nump + 1, np.int64)
    es[1:] = np.cumsum(counts)
    pos = rng.uniform(-0.5 * E, 0.5 * E, size=(int(es[-1]), 3))
    return pids, es, np.ascontiguousarray(pos)


@pytest.mark.parametrize("bc", ["pbc", "free_space"])
def test_noalloc_matches_allocating_entry_point(bc):
    import torch
    from coulomb_kmc_gb300 import KMCFMM, _native
    from coulomb_kmc_gb300.dats import make_state

    lib = _native.lib()
    E, N = 6.0, 300
    rng = np.random.default_rng(21)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    st = make_state(P, neutral_charges(N), E)
    k = KMCFMM(st.P, st.Q, st.domain, r=3, l=12, boundary_condition=bc)
    k.initialise()
    for call in range(2):
        pids, es, pos = _moves(rng, N, E, nump=60 + 40 * call, max_k=5)
        total = int(es[-1])
        ref = np.zeros(total)
        _native.check(lib.kmc_propose_moves(k._handle, len(pids), pids.ctypes.data, es.ctypes.data,
                                            pos.ctypes.data, ref.ctypes.data), "kmc_propose_moves")
        d_pids = torch.from_numpy(pids).cuda()
        d_es = torch.from_numpy(es).cuda()
        d_pos = torch.from_numpy(pos).cuda()
        d_out = torch.full((total,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        k._set_stream()
        rc = lib.kmc_propose_moves_noalloc(k._handle, len(pids), total, d_pids.data_ptr(), d_es.data_ptr(),
                                           d_pos.data_ptr(), d_out.data_ptr())
        _native.check(rc, "kmc_propose_moves_noalloc")
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.max(rel_err(got, ref)) < TOL
    k.free()


def test_noalloc_rejects_oversized_calls():
    import torch
    from coulomb_kmc_gb300 import KMCFMM, _native
    from coulomb_kmc_gb300.dats import make_state

    lib = _native.lib()
    E, N = 4.0, 64
    rng = np.random.default_rng(3)
    st = make_state(rng.uniform(-0.5 * E, 0.5 * E, (N, 3)), neutral_charges(N), E)
    k = KMCFMM(st.P, st.Q, st.domain, r=2, l=6, boundary_condition="27")
    k.initialise()
    buf = torch.zeros(8, dtype=torch.int64, device="cuda")
    rc = lib.kmc_propose_moves_noalloc(k._handle, 1, 16385, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                                       buf.data_ptr())
    assert rc == -1
    assert b"16384" in lib.kmc_last_error()
    rc = lib.kmc_propose_moves_noalloc(k._handle, 4097, 4097, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                                       buf.data_ptr())
    assert rc == -1
    k.free()
