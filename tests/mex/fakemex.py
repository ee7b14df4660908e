"""Builds the MEX gateway (mnad-modeling-rtm_gb300/matlab/mnad_mex.c) against
the fake MATLAB API of this directory and libmnad.so, and calls it the way
MATLAB would: ``call('fwd', dx, xs, ...)`` with numpy arrays and scalars as
the right-hand side.  Test infrastructure only."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
GATEWAY = os.path.join(ROOT, "mnad-modeling-rtm_gb300", "matlab", "mnad_mex.c")
OUT = os.path.join(HERE, "_build", "libfakemex.so")

_L = None


class MexError(RuntimeError):
    def __init__(self, ident, msg):
        self.identifier = ident
        super().__init__(f"{ident}: {msg}")


def build():
    from mnad import _lib, build as libbuild
    libbuild.build()
    libdir = os.path.dirname(_lib.LIB_PATH)
    deps = [GATEWAY, os.path.join(HERE, "fake_mx.c"), os.path.join(HERE, "mex.h"), _lib.LIB_PATH,
            os.path.join(ROOT, "include", "mnad.h")]
    if not os.path.exists(OUT) or any(os.path.getmtime(d) > os.path.getmtime(OUT) for d in deps):
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-shared", "-fPIC", "-I", HERE,
                        "-I", os.path.join(ROOT, "include"), GATEWAY, os.path.join(HERE, "fake_mx.c"),
                        "-L", libdir, "-l:libmnad.so", "-Wl,-rpath," + libdir, "-o", OUT], check=True)
    return OUT


def lib():
    global _L
    if _L is None:
        from mnad import _lib
        _lib.lib()                      # the same libmnad.so instance as the Python binding
        L = C.CDLL(build())
        vp = C.c_void_p
        L.fmx_double.argtypes = [C.c_size_t, C.c_size_t, C.POINTER(C.c_double)]
        L.fmx_double.restype = vp
        L.fmx_string.argtypes = [C.c_char_p]
        L.fmx_string.restype = vp
        L.fmx_cell1.argtypes = [vp]
        L.fmx_cell1.restype = vp
        L.fmx_kind.argtypes = [vp]
        L.fmx_call.argtypes = [C.c_int, C.POINTER(vp), C.c_int, C.POINTER(vp)]
        L.fmx_error_id.restype = C.c_char_p
        L.fmx_error_msg.restype = C.c_char_p
        for n in ("mxGetPr",):
            getattr(L, n).argtypes = [vp]
            getattr(L, n).restype = C.POINTER(C.c_double)
        for n in ("mxGetM", "mxGetN"):
            getattr(L, n).argtypes = [vp]
            getattr(L, n).restype = C.c_size_t
        L.mxGetCell.argtypes = [vp, C.c_size_t]
        L.mxGetCell.restype = vp
        _L = L
    return _L


def _arg(x):
    L = lib()
    if isinstance(x, str):
        return L.fmx_string(x.encode())
    if isinstance(x, list):                        # a 1x1 cell
        return L.fmx_cell1(_arg(x[0]))
    a = np.asarray(x, dtype=np.float64)
    if a.ndim == 0:
        a = a.reshape(1, 1)
    elif a.ndim == 1:
        a = a.reshape(1, -1)                       # row vector, as MATLAB's xr/zr
    a = np.asfortranarray(a)
    return L.fmx_double(a.shape[0], a.shape[1], a.ctypes.data_as(C.POINTER(C.c_double)))


def _out(p):
    L = lib()
    kind = L.fmx_kind(p)
    if kind == 1:
        return [_out(L.mxGetCell(p, 0))]
    m, n = L.mxGetM(p), L.mxGetN(p)
    pr = L.mxGetPr(p)
    return np.ctypeslib.as_array(pr, shape=(m * n,)).reshape((m, n), order="F").copy()


def call(cmd, *args, nlhs=1):
    L = lib()
    rhs = (C.c_void_p * (len(args) + 1))(*([_arg(cmd)] + [_arg(a) for a in args]))
    lhs = (C.c_void_p * max(nlhs, 1))()
    if L.fmx_call(nlhs, lhs, len(args) + 1, rhs):
        raise MexError(L.fmx_error_id().decode(), L.fmx_error_msg().decode())
    outs = [_out(lhs[k]) for k in range(nlhs) if lhs[k]]
    return outs[0] if nlhs == 1 and outs else outs


def at_exit():
    lib().fmx_exit()
