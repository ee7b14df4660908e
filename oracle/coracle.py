"""ctypes front end of the C oracle (test infrastructure only).

Same conventions as ``oracle/mnad_oracle.py``: arrays of MATLAB shape
``(nz, nx)``, 1-based source/receiver indices, FP64.  Results are returned as
NumPy arrays.  The library is built by ``oracle/build_oracle.py``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.LIB
        if not os.path.exists(path):
            path = build_oracle.build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.mnad_oracle_fwd.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                      dp, C.c_int, C.c_int, C.c_int, ip, ip, C.c_int, dp, C.c_int,
                                      C.c_int, C.c_int, dp, dp, dp, dp, dp, C.c_int, ip, dp]
        L.mnad_oracle_fwd.restype = C.c_int
        L.mnad_oracle_adj.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                      dp, C.c_int, ip, ip, C.c_int, dp, dp, C.c_int, C.c_int,
                                      C.c_int, dp]
        L.mnad_oracle_adj.restype = C.c_int
        L.mnad_oracle_threads.restype = C.c_int
        _lib = L
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


def threads() -> int:
    return lib().mnad_oracle_threads()


def fwd(dx, xs, xr, dz, zs, zr, v, dt, nt, w, d_pml, indx=0, T=1, ncols=0,
        record_vw=False, keep_steps=()):
    """Forward shot; returns dict(datau[, datav, dataw][, UU, illum][, fields])."""
    v = np.asfortranarray(v, dtype=np.float64)
    nz, nx = v.shape
    xr = np.ascontiguousarray(np.asarray(xr).ravel(), dtype=np.int32)
    zr = np.ascontiguousarray(np.asarray(zr).ravel(), dtype=np.int32)
    nr = xr.size
    w = np.ascontiguousarray(np.asarray(w, dtype=np.float64).ravel())
    datau = np.zeros((nt, nr), order="F")
    datav = np.zeros((nt, nr), order="F") if record_vw else None
    dataw = np.zeros((nt, nr), order="F") if record_vw else None
    d = d_pml
    UU = illum = None
    if indx == 1:
        nint = (nz - 2 * d) * (nx - 2 * d)
        UU = np.zeros((nint, ncols), order="F")
        illum = np.zeros((nz - 2 * d, nx - 2 * d), order="F")
    keep = np.ascontiguousarray(np.asarray(keep_steps, dtype=np.int32))
    N = nz * nx
    keep_out = np.zeros(max(1, keep.size) * 3 * N)
    rc = lib().mnad_oracle_fwd(nz, nx, dz, dx, dt, d, _d(v), int(zs), int(xs), nr, _i(zr), _i(xr),
                               nt, _d(w), indx, T, ncols, _d(datau), _d(datav), _d(dataw), _d(UU),
                               _d(illum), keep.size, _i(keep) if keep.size else None, _d(keep_out))
    if rc != 0:
        raise ValueError("mnad_oracle_fwd rejected its arguments")
    out = {"datau": datau}
    if record_vw:
        out["datav"], out["dataw"] = datav, dataw
    if indx == 1:
        out["UU"], out["illum"] = UU, illum
    out["fields"] = {int(t): tuple(keep_out[(k * 3 + f) * N:(k * 3 + f + 1) * N].reshape((nz, nx), order="F")
                                   for f in range(3)) for k, t in enumerate(keep)}
    return out


def adj(dx, dz, nt, dt, v, xr, zr, data, d_pml, UU, T, pairing="reference"):
    """Adjoint shot + imaging; returns Im (Nint,)."""
    v = np.asfortranarray(v, dtype=np.float64)
    nz, nx = v.shape
    if isinstance(data, (list, tuple)):
        data = data[0]
    data = np.asfortranarray(data, dtype=np.float64)
    xr = np.ascontiguousarray(np.asarray(xr).ravel(), dtype=np.int32)
    zr = np.ascontiguousarray(np.asarray(zr).ravel(), dtype=np.int32)
    UU = np.asfortranarray(UU, dtype=np.float64)
    nint = (nz - 2 * d_pml) * (nx - 2 * d_pml)
    Im = np.zeros(nint)
    rc = lib().mnad_oracle_adj(nz, nx, dz, dx, dt, d_pml, _d(v), xr.size, _i(zr), _i(xr), nt, _d(data),
                               _d(UU), UU.shape[1], T, 0 if pairing == "reference" else 1, _d(Im))
    if rc != 0:
        raise ValueError("mnad_oracle_adj rejected its arguments")
    return Im
