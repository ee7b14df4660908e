"""ctypes binding of libmnad.so (the C ABI declared in include/mnad.h).

The binding is thin on purpose: every call goes straight to the CUDA
library.  There is no CPU fallback -- if the library is missing or no GPU is
present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmnad.so")

# Status codes (include/mnad.h).
OK, E_ARG, E_OOM, E_CUDA, E_TIMEOUT, E_NOTFOUND, E_NUMERIC, E_BUDGET, E_STATE = range(9)
SNAP_F32, SNAP_BF16, SNAP_F16 = 0, 1, 2
PAIR_REFERENCE, PAIR_ALIGNED = 0, 1
KERNEL_AUTO, KERNEL_DIRECT, KERNEL_TMA, KERNEL_TUNE, KERNEL_TMA2, KERNEL_TMA_NARROW = 0, 1, 2, 3, 4, 5
JOB_MODEL, JOB_RTM = 0, 1
JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3

_CODE_NAMES = {E_ARG: "arg", E_OOM: "oom", E_CUDA: "cuda", E_TIMEOUT: "timeout", E_NOTFOUND: "notfound",
               E_NUMERIC: "numeric", E_BUDGET: "budget", E_STATE: "state"}

# Every function the header declares, with its ctypes signature.
_dp = C.POINTER(C.c_double)
_vp = C.c_void_p


class Options(C.Structure):
    _fields_ = [("snapshot_codec", C.c_int), ("pairing", C.c_int), ("T", C.c_int),
                ("record_vw", C.c_int), ("use_graphs", C.c_int), ("kernel", C.c_int),
                ("energy_every", C.c_int), ("checkpoint_every", C.c_int), ("checkpoint_codec", C.c_int)]


class Job(C.Structure):
    _fields_ = [("kind", C.c_int), ("nz", C.c_int), ("nx", C.c_int), ("d_pml", C.c_int), ("nt", C.c_int),
                ("dx", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
                ("v", _dp), ("vs", _dp), ("zs", C.c_double), ("xs", C.c_double),
                ("nr", C.c_int), ("zr", _dp), ("xr", _dp), ("w", _dp), ("T", C.c_int),
                ("data_out", _dp), ("image_out", _dp), ("illum_out", _dp)]


class ServerOptions(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("chunk_steps", C.c_int), ("max_active_jobs", C.c_int),
                ("snapshot_codec", C.c_int), ("kernel", C.c_int), ("no_graphs", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64), ("queued", C.c_int64),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double),
                ("point_updates", C.c_double), ("busy_s", C.c_double), ("wall_s", C.c_double),
                ("bytes_in_use", C.c_size_t), ("peak_bytes", C.c_size_t)]


SIGNATURES = {
    "mnad_abi_version": ([], C.c_int),
    "mnad_last_error": ([], C.c_char_p),
    "mnad_context_create": ([C.c_int, C.c_size_t, C.POINTER(_vp)], C.c_int),
    "mnad_context_destroy": ([_vp], C.c_int),
    "mnad_context_set_options": ([_vp, C.POINTER(Options)], C.c_int),
    "mnad_context_get_options": ([_vp, C.POINTER(Options)], C.c_int),
    "mnad_context_memory": ([_vp, C.POINTER(C.c_size_t)], C.c_int),
    "mnad_context_status": ([_vp, C.POINTER(C.c_uint)], C.c_int),
    "mnad_context_set_wait_limit": ([_vp, C.c_uint], C.c_int),
    "mnad_context_energy": ([_vp, _dp, C.c_int, C.POINTER(C.c_int)], C.c_int),
    "mnad_context_transfers": ([_vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], C.c_int),
    "mnad_fwd_pde_exact": ([_vp, C.c_double, C.c_double, _dp, C.c_int, C.c_double, C.c_double, _dp,
                            _dp, C.c_int, C.c_int, C.c_double, C.c_int, _dp, C.c_int, C.c_int, C.c_int,
                            _dp, _dp, _dp], C.c_int),
    "mnad_fwd_fields": ([_vp, C.c_double, C.c_double, _dp, C.c_int, C.c_double, C.c_double, _dp,
                         _dp, C.c_int, C.c_int, C.c_double, C.c_int, _dp, C.c_int, C.c_int,
                         C.POINTER(C.c_int), _dp, _dp], C.c_int),
    "mnad_fwd_pde_exact_noalloc": ([C.c_int, C.c_double, C.c_double, _dp, C.c_int, C.c_double, C.c_double, _dp,
                                    _dp, C.c_int, C.c_int, C.c_double, C.c_int, _dp, C.c_int, _dp], C.c_int),
    "mnad_born_adj": ([_vp, C.c_double, C.c_double, C.c_int, C.c_double, _dp, C.c_int, C.c_int, _dp, _dp,
                       C.c_int, _dp, C.c_int, C.c_int, _dp], C.c_int),
    "mnad_wavefield_info": ([_vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int), C.POINTER(C.c_int),
                             C.POINTER(C.c_int)], C.c_int),
    "mnad_wavefield_export": ([_vp, C.c_int, _dp, _dp], C.c_int),
    "mnad_wavefield_import": ([_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                               _dp, _dp], C.c_int),
    "mnad_wavefield_release": ([_vp, C.c_int], C.c_int),
    "mnad_run_jobs": ([_vp, C.POINTER(Job), C.c_int], C.c_int),
    "mnad_plan_create": ([_vp, C.POINTER(Job), C.c_int, C.POINTER(_vp)], C.c_int),
    "mnad_plan_run": ([_vp], C.c_int),
    "mnad_plan_download": ([_vp], C.c_int),
    "mnad_plan_destroy": ([_vp], C.c_int),
    "mnad_plan_work": ([_vp, _dp, _dp], C.c_int),
    "mnad_plan_timing": ([_vp, _dp, _dp, C.POINTER(C.c_int)], C.c_int),
    "mnad_plan_phases": ([_vp, _dp, _dp, _dp, _dp], C.c_int),
    "mnad_plan_kernels": ([_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
    "mnad_plan_stack": ([_vp, _dp, _dp, _dp], C.c_int),
    "mnad_server_create": ([C.c_int, C.POINTER(ServerOptions), C.POINTER(_vp)], C.c_int),
    "mnad_server_submit": ([_vp, C.POINTER(Job), C.POINTER(C.c_uint64)], C.c_int),
    "mnad_server_poll": ([_vp, C.c_uint64, C.POINTER(C.c_int)], C.c_int),
    "mnad_server_wait": ([_vp, C.c_uint64, C.c_double], C.c_int),
    "mnad_server_get_stats": ([_vp, C.POINTER(ServerStats)], C.c_int),
    "mnad_server_destroy": ([_vp], C.c_int),
}


class MnadError(RuntimeError):
    """A non-zero status of the C ABI; ``identifier`` mirrors MATLAB's error ids."""

    def __init__(self, code: int, message: str):
        self.code = code
        self.identifier = "mnad:" + _CODE_NAMES.get(code, str(code))
        super().__init__(f"{self.identifier}: {message}")


_lib = None


def lib():
    """Load libmnad.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with mnad.build.build() "
                              "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != OK:
        msg = lib().mnad_last_error()
        raise MnadError(rc, msg.decode() if msg else "")
