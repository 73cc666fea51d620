"""The allocation-free entry point kmc_propose_moves_noalloc.

Some callers of this library cannot allocate device memory when they need
energy differences: an application whose own memory pool has already claimed
the device memory it is allowed to use (a molecular-dynamics engine or a
framework's caching allocator, where a cudaMalloc from a library fails or
fragments the pool), or a tight loop where a cudaMalloc / cudaFree pair would
stall the device (cudaFree synchronises it).  This entry point keeps its
scratch in a fixed device array inside the library; the caller passes only
inputs and outputs, in device memory.

The tests call it through the C ABI two times in a row with different moves and
check each result against the allocating entry point kmc_propose_moves at the
1e-10 tolerance of the other parity tests, for every boundary condition and for
an expansion order above 16 (another shared-memory size); then they check that
invalid ids, offsets and positions are answered with NaN and an error count,
never with a read outside the buffers, and that the next call is correct again.
The file is named so that pytest collects it last.
"""
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


def _system(bc, L, N=300, E=6.0, seed=21, R=3):
    from coulomb_kmc_gb300 import KMCFMM
    from coulomb_kmc_gb300.dats import make_state
    rng = np.random.default_rng(seed)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    st = make_state(P, neutral_charges(N), E)
    k = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition=bc)
    k.initialise()
    return k, rng


def _noalloc(k, pids, es, pos, total=None):
    import torch
    from coulomb_kmc_gb300 import _native
    total = int(es[-1]) if total is None else int(total)
    d_pids = torch.from_numpy(np.ascontiguousarray(pids)).cuda()
    d_es = torch.from_numpy(np.ascontiguousarray(es)).cuda()
    d_pos = torch.from_numpy(np.ascontiguousarray(pos)).cuda()
    d_out = torch.zeros((max(total, 1),), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    k._set_stream()
    rc = _native.lib().kmc_propose_moves_noalloc(k._handle, len(pids), total, d_pids.data_ptr(), d_es.data_ptr(),
                                                 d_pos.data_ptr(), d_out.data_ptr())
    _native.check(rc, "kmc_propose_moves_noalloc")
    torch.cuda.synchronize()
    return d_out.cpu().numpy()[:total]


def _allocating(k, pids, es, pos):
    from coulomb_kmc_gb300 import _native
    ref = np.zeros(int(es[-1]))
    _native.check(_native.lib().kmc_propose_moves(k._handle, len(pids), pids.ctypes.data, es.ctypes.data,
                                                  pos.ctypes.data, ref.ctypes.data), "kmc_propose_moves")
    return ref


@pytest.mark.parametrize("bc,L", [("pbc", 12), ("free_space", 12), ("27", 12), ("pbc", 20)])
def test_noalloc_matches_allocating_entry_point(bc, L):
    k, rng = _system(bc, L)
    for call in range(2):
        pids, es, pos = _moves(rng, k.N, 6.0, nump=60 + 40 * call, max_k=5)
        ref = _allocating(k, pids, es, pos)
        got = _noalloc(k, pids, es, pos)
        assert np.all(np.isfinite(got))
        assert np.max(rel_err(got, ref)) < TOL
    assert k.error_counts() == (0, 0)
    k.free()


def test_noalloc_rejects_invalid_inputs_without_reading_past_buffers():
    k, rng = _system("pbc", 12, N=200, E=5.0)
    N = k.N
    pids, es, pos = _moves(rng, N, 5.0, nump=20, max_k=3)
    total = int(es[-1])
    # ids out of range: every output NaN, one bad call counted
    for bad_pid in (N, N + 1000, -1):
        p2 = pids.copy()
        p2[7] = bad_pid
        out = _noalloc(k, p2, es, pos)
        assert np.all(np.isnan(out))
        assert k.error_counts()[0] == 1
    # offsets that do not start at 0, decrease, or end elsewhere than `total`
    for mutate in ("start", "decrease", "end"):
        e2 = es.copy()
        if mutate == "start":
            e2[0] = 1
        elif mutate == "decrease":
            e2[5] = e2[4] - 1
        else:
            e2[-1] = total + 3
        out = _noalloc(k, pids, e2, pos, total=total)
        assert np.all(np.isnan(out))
        assert k.error_counts()[0] == 1
    # positions outside the box or not finite: only those proposals are NaN
    p3 = pos.copy()
    p3[2, 0] = 2.6          # beyond +E/2
    p3[5, 1] = -9.0         # beyond -E/2
    p3[8, 2] = np.nan
    out = _noalloc(k, pids, es, p3)
    ref = _allocating(k, pids, es, pos)
    badrows = np.array([2, 5, 8])
    assert np.all(np.isnan(out[badrows]))
    good = np.setdiff1d(np.arange(total), badrows)
    assert np.max(rel_err(out[good], ref[good])) < TOL
    assert k.error_counts()[0] == 3
    # the context stays usable and the next call is correct
    out = _noalloc(k, pids, es, pos)
    assert np.max(rel_err(out, ref)) < TOL
    assert k.error_counts() == (0, 0)
    k.free()


def test_noalloc_rejects_oversized_calls():
    import torch
    from coulomb_kmc_gb300 import _native

    lib = _native.lib()
    k, _ = _system("27", 6, N=64, E=4.0, seed=3, R=2)
    buf = torch.zeros(8, dtype=torch.int64, device="cuda")
    rc = lib.kmc_propose_moves_noalloc(k._handle, 1, 16385, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                                       buf.data_ptr())
    assert rc == -1
    assert b"16384" in lib.kmc_last_error()
    rc = lib.kmc_propose_moves_noalloc(k._handle, 4097, 4097, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                                       buf.data_ptr())
    assert rc == -1
    k.free()
