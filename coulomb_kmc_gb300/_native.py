"""Build and load libkmc_gb300.so (the C ABI declared in include/kmc_gb300.h).

The library is compiled in-tree for sm_103a with nvcc.  There is no CPU
fallback: if the library cannot be built or loaded, every entry point raises.
"""
import ctypes
import os
import shutil
import subprocess
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_void_p

_PKG = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_PKG)
BUILD_DIR = os.path.join(_PKG, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libkmc_gb300.so")
SOURCES = [os.path.join(_PKG, "csrc", "kmc_gb300.cu"), os.path.join(_PKG, "csrc", "kmc_driver.cu")]

def _deps():
    """Every source the library is built from: the translation units, every
    header and fragment in csrc/ and the public header."""
    csrc = os.path.join(_PKG, "csrc")
    extra = sorted(os.path.join(csrc, n) for n in os.listdir(csrc) if n.endswith((".cuh", ".h", ".inc")))
    return SOURCES + extra + [os.path.join(_ROOT, "include", "kmc_gb300.h")]


DEPS = _deps()
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]

KMC_BC = {"free_space": 0, "27": 1, "pbc": 2}
KMC_PREC = {"fp64": 0, "mixed": 1, "mixed_fp64_accept": 2}
KMC_INIT = {"auto": 0, "exact": 1, "fmm": 2}
KMC_ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "not initialised", -4: "bad proposed move",
              -5: "cell store overflow", -6: "out of memory"}


class KmcParams(ctypes.Structure):
    _fields_ = [
        ("boundary", c_int32), ("r", c_int32), ("l", c_int32), ("precision", c_int32),
        ("extent", c_double), ("max_move", c_double), ("energy_unit", c_double),
        ("lr_nnz", c_int64), ("lr_data", POINTER(c_double)), ("lr_indptr", POINTER(c_int64)),
        ("lr_indices", POINTER(c_int64)), ("lr_dipole", c_double * 3), ("initial_solve", c_int32),
    ]


class KmcDriverParams(ctypes.Structure):
    _fields_ = [
        ("kind", c_int32), ("lattice_side", c_int32), ("beta", c_double), ("step", c_double),
        ("seed", ctypes.c_uint64), ("lattice_sites", POINTER(c_int64)), ("log_capacity", c_int64),
    ]


KMC_DRIVE = {"lattice": 0, "offlattice": 1}
# tuning keys (include/kmc_gb300.h)
KMC_TUNE_P2L_GROUPS = 0
KMC_TUNE_LR_FUSED = 1
KMC_TUNE_LR_STAGE = 2
KMC_TUNE_NEAR_SCALAR = 3
KMC_TUNE_NEAR_CHUNK = 4
KMC_TUNE_LR_NOCACHE = 5
KMC_TUNE_P2L_FP32_FROM = 6
KMC_TUNE_DRIVER_SERIAL = 7
KMC_TUNE_FSELF_GENERIC = 8
KMC_TUNE_P2L_PAIR = 9
KMC_TUNE_P2L64 = 10
KMC_TUNE_P2L64_CELLS = 11
KMC_TUNE_LR_THREADS = 12
KMC_TUNE_NEAR_SPLIT = 13
KMC_TUNE_NEAR_OLD = 14
KMC_TUNE_P2L64_PER_SM = 15
KMC_TUNE_NEAR_PRIORITY = 16


def _nvcc():
    nv = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nv):
        raise RuntimeError("nvcc not found: the CUDA library cannot be built")
    return nv


def build(force=False, verbose=False):
    """Compile libkmc_gb300.so for sm_103a (no GPU needed)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH):
        lib_m = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= lib_m for d in DEPS):
            return LIB_PATH
    tmp = LIB_PATH + ".tmp"
    cmd = [_nvcc(), *ARCH_FLAGS, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-I" + os.path.join(_ROOT, "include"), "-o", tmp, *SOURCES]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + r.stdout + r.stderr)
    if verbose:
        print(r.stdout + r.stderr)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None

# every exported symbol with its ctypes signature (argtypes, restype)
SIGNATURES = {
    "kmc_create": ([POINTER(KmcParams), POINTER(c_void_p)], c_int),
    "kmc_set_stream": ([c_void_p, c_void_p], c_int),
    "kmc_initialise": ([c_void_p, c_int64, c_void_p, c_void_p, POINTER(c_double)], c_int),
    "kmc_propose_with_dats": ([c_void_p, c_int64, c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                               c_void_p, c_void_p], c_int),
    "kmc_propose_moves": ([c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p], c_int),
    "kmc_accept": ([c_void_p, c_int64, POINTER(c_double)], c_int),
    "kmc_accept_device": ([c_void_p, c_void_p, c_void_p, c_void_p], c_int),
    "kmc_propose_moves_noalloc": ([c_void_p, c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p], c_int),
    "kmc_get_energy": ([c_void_p, POINTER(c_double)], c_int),
    "kmc_get_error": ([c_void_p, POINTER(c_int64), POINTER(c_int64)], c_int),
    "kmc_store_reserve": ([c_void_p, c_int64], c_int),
    "kmc_max_occupancy": ([c_void_p, POINTER(c_int64), POINTER(c_int64)], c_int),
    "kmc_resolve_overflow": ([c_void_p, POINTER(c_int64)], c_int),
    "kmc_read_state": ([c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p], c_int),
    "kmc_info": ([c_void_p, POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)], c_int),
    "kmc_profile": ([c_void_p, c_int32], c_int),
    "kmc_profile_read": ([c_void_p, c_int32, c_void_p, c_void_p, POINTER(c_int64)], c_int),
    "kmc_profile_timeline": ([c_void_p, c_int64, c_void_p, c_void_p, c_void_p, POINTER(c_int64)], c_int),
    "kmc_kernel_name": ([c_int32], c_char_p),
    "kmc_eval_field": ([c_void_p, c_int64, c_void_p, c_void_p], c_int),
    "kmc_get_energy_ids": ([c_void_p, c_int64, c_void_p, c_void_p], c_int),
    "kmc_group_energy": ([c_void_p, c_int64, c_void_p, c_void_p, c_void_p], c_int),
    "kmc_extract": ([c_void_p, c_int64, c_void_p, POINTER(c_double)], c_int),
    "kmc_inject": ([c_void_p, c_int64, c_void_p, c_void_p, POINTER(c_double)], c_int),
    "kmc_set_tuning": ([c_void_p, c_int32, c_int32], c_int),
    "kmc_get_tuning": ([c_void_p, c_int32, POINTER(c_int32)], c_int),
    "kmc_autotune": ([c_void_p, c_int32, c_void_p], c_int),
    "kmc_bucket_create": ([c_void_p, c_int64, POINTER(c_void_p)], c_int),
    "kmc_bucket_launch": ([c_void_p, c_int64, c_void_p], c_int),
    "kmc_bucket_free": ([c_void_p], c_int),
    "kmc_driver_create": ([c_void_p, POINTER(KmcDriverParams), POINTER(c_void_p)], c_int),
    "kmc_driver_step": ([c_void_p, c_int64], c_int),
    "kmc_driver_capture": ([c_void_p], c_int),
    "kmc_driver_launch": ([c_void_p, c_int64, c_void_p], c_int),
    "kmc_driver_counters": ([c_void_p, POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)], c_int),
    "kmc_driver_log": ([c_void_p, c_int64, c_void_p, c_void_p, c_void_p, POINTER(c_int64)], c_int),
    "kmc_driver_sites": ([c_void_p, c_void_p], c_int),
    "kmc_driver_free": ([c_void_p], c_int),
    "kmc_drivers_launch": ([c_void_p, c_int64, c_int64, c_void_p, c_void_p, c_int64], c_int),
    "kmc_stream_create": ([POINTER(c_void_p)], c_int),
    "kmc_stream_destroy": ([c_void_p], c_int),
    "kmc_propose_with_dats_host": ([c_void_p, c_int64, c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, POINTER(c_int64)], c_int),
    "kmc_host_displacements": ([c_int64, c_void_p, c_double, c_double, ctypes.c_uint64, c_int64, c_void_p, c_int32],
                               c_int),
    "kmc_diag_fma_rate": ([c_int32, c_int32, POINTER(c_double)], c_int),
    "kmc_free": ([c_void_p], c_int),
    "kmc_last_error": ([], c_char_p),
}


def lib():
    """Load the library (building it first if needed); raises if unavailable."""
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        for name, (argt, rest) in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = argt
            f.restype = rest
        _lib = L
    return _lib


class DedicatedStream:
    """A CUDA stream of its own (kmc_stream_create), usable as a torch stream.
    torch.cuda.Stream() hands out streams from a fixed pool round-robin, so two of
    them can be one CUDA stream; a step captured on one while another thread
    launches on its alias fails.  Drivers and the server use these instead."""

    def __init__(self):
        import torch
        h = c_void_p()
        check(lib().kmc_stream_create(ctypes.byref(h)), "kmc_stream_create")
        self.handle = h
        self.stream = torch.cuda.ExternalStream(h.value)

    @property
    def cuda_stream(self):
        return self.handle.value

    def close(self):
        if self.handle is not None and self.handle.value:
            check(lib().kmc_stream_destroy(self.handle), "kmc_stream_destroy")
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


NKERNELS = 19
NTUNE = 17


def check(rc, what):
    if rc != 0:
        msg = lib().kmc_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed: {KMC_ERRORS.get(rc, rc)} ({msg})")
