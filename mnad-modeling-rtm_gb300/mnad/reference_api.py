"""Drop-in mirrors of the reference's two propagator functions.

``fwd_PDE_exact_MNAD`` and ``Born_adj_MNAD`` keep the MATLAB argument lists of
``SRC/MNAD/fwd_PDE_exact_MNAD.m:1`` and ``SRC/migration/Born_adj_MNAD.m:1``
(argument order, meaning, 1-based padded indices, the ignored-but-accepted
sparse operators, the ``indx`` flag) and their return values (a one-element
list standing for the 1x1 cell ``data``; an ``Nint x 1`` column for ``Im``).
The on-disk hand-off ``./Wavefields/UU_<ss>.mat`` becomes device storage
keyed by ``ss`` inside a :class:`mnad.api.Context`; ``save_wavefield`` /
``load_wavefield`` write and read the same ``.mat`` files when a shot's
forward and adjoint run in different processes.
"""
from __future__ import annotations

import os

import numpy as np

from .api import Context

_default_ctx = None

# A MAT v5 data element stores its size in 32 bits and MATLAB reads variables
# of at most 2 GiB from such files; larger ones need the HDF5-based v7.3
# format, which this module does not write.
MAT_V5_MAX_BYTES = 2 ** 31 - 1


def _payload_bytes(x) -> int:
    if isinstance(x, dict):
        return sum(_payload_bytes(v) for v in x.values())
    a = np.asarray(x)
    if a.dtype == object:
        return sum(_payload_bytes(v) for v in a.ravel())
    return a.nbytes


def _savemat(path: str, variables: dict):
    """scipy.io.savemat in MAT v5, refusing variables MATLAB could not read
    back (over 2 GiB) instead of writing a broken file."""
    import scipy.io
    for name, val in variables.items():
        n = _payload_bytes(val)
        if n > MAT_V5_MAX_BYTES:
            raise ValueError(f"variable '{name}' holds {n} bytes: MAT v5 files keep at most {MAT_V5_MAX_BYTES} "
                             "bytes per variable; keep it on the device (mnad_wavefield_*) or write it in parts")
    scipy.io.savemat(path, variables, format="5")


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def fwd_PDE_exact_MNAD(dx, xs, xr, dz, zs, zr, v, dt, nt, w, d_pml, ss,
                       Auu=None, Auv=None, Auw=None, Avu=None, Avv=None, Avw=None,
                       Awu=None, Awv=None, Aww=None, indx=0, *, ctx: Context | None = None):
    """Forward modeling of one shot; returns ``[datau]`` (nt x nr).

    The nine sparse operators are accepted for signature compatibility and
    ignored: the device recomputes the same coefficients from ``v``.  With
    ``indx=1`` the d2u snapshots and illumination stay on the GPU under shot
    id ``ss`` (see :meth:`Context.wavefield_export`).
    """
    ctx = ctx or default_context()
    datau = ctx.fwd(dx, xs, xr, dz, zs, zr, v, dt, nt, w, d_pml, ss=ss, indx=0 if indx is None else indx)
    return [datau]


def Born_adj_MNAD(dx, dz, nt, dt, v, xr, zr, data, d_pml, ss,
                  Auu=None, Auv=None, Auw=None, Avu=None, Avv=None, Avw=None,
                  Awu=None, Awv=None, Aww=None, *, ctx: Context | None = None):
    """Reverse-time propagation + imaging of one shot; returns ``Im`` (Nint x 1).

    ``data`` may be the cell returned by the forward (a list: ``data[0]`` is
    used, as ``data{1}`` at ``Born_adj_MNAD.m:50``) or an ``nt x nr`` array
    (what the reference driver actually passes, ``main_Acoustic_RTM.m:248``).
    """
    ctx = ctx or default_context()
    im = ctx.adj(dx, dz, nt, dt, v, xr, zr, data, d_pml, ss=ss)
    return im.reshape(-1, 1, order="F")


def save_wavefield(ctx: Context, ss: int, nz: int, nx: int, d_pml: int, directory: str = "."):
    """Write ``Wavefields/UU_<ss>.mat`` and ``Illuminations/illum_<ss>.mat``
    (variables ``UU`` and ``illum``) as ``fwd_PDE_exact_MNAD.m:160-164`` does."""
    info = ctx.wavefield_info(ss)
    if info["nint"] * info["ncols"] * 8 > MAT_V5_MAX_BYTES:
        raise ValueError(f"UU of shot {ss} holds {info['nint'] * info['ncols'] * 8} bytes: MAT v5 files keep at most "
                         f"{MAT_V5_MAX_BYTES} bytes per variable; keep it on the device (mnad_wavefield_*)")
    UU, illum = ctx.wavefield_export(ss)
    os.makedirs(os.path.join(directory, "Wavefields"), exist_ok=True)
    os.makedirs(os.path.join(directory, "Illuminations"), exist_ok=True)
    _savemat(os.path.join(directory, "Wavefields", f"UU_{ss}.mat"), {"UU": UU})
    _savemat(os.path.join(directory, "Illuminations", f"illum_{ss}.mat"),
             {"illum": illum.reshape((nz - 2 * d_pml, nx - 2 * d_pml), order="F")})


def load_wavefield(ctx: Context, ss: int, nz: int, nx: int, d_pml: int, nt: int, T: int, directory: str = "."):
    """Read ``Wavefields/UU_<ss>.mat`` back into device storage for shot ``ss``
    (the ``load`` at ``Born_adj_MNAD.m:33``).  Trailing all-zero columns of
    the reference's preallocated matrix stay part of ``ncols``.  The
    illumination written beside it is stored with it when present."""
    import scipy.io
    UU = scipy.io.loadmat(os.path.join(directory, "Wavefields", f"UU_{ss}.mat"))["UU"]
    illum = None
    ipath = os.path.join(directory, "Illuminations", f"illum_{ss}.mat")
    if os.path.exists(ipath):
        illum = scipy.io.loadmat(ipath)["illum"].ravel(order="F")
    nsnap = nt // T
    ctx.wavefield_import(ss, nz, nx, d_pml, nt, T, UU, nsnap=min(nsnap, UU.shape[1]), illum=illum)


# Fields of the drivers' ``profile`` struct (SRC/migration/main_Acoustic_RTM.m:64-132,
# SRC/modeling/main_Acoustic_Data.m), in the order the drivers set them.
PROFILE_FIELDS = ("fc", "f_max", "dt", "T_max", "dx", "nx", "dz", "nz", "ns")


def make_profile(fc, dt, T_max, dx, nx, dz, nz, ns, f_max=None) -> dict:
    """The drivers' ``profile`` struct as a dict (``f_max = 3 fc`` by default,
    main_Acoustic_RTM.m:62)."""
    return {"fc": float(fc), "f_max": float(3.0 * fc if f_max is None else f_max), "dt": float(dt),
            "T_max": float(T_max), "dx": float(dx), "nx": float(nx), "dz": float(dz), "nz": float(nz),
            "ns": float(ns)}


def _cell_row(items):
    """A 1 x n MATLAB cell array for scipy.io.savemat."""
    c = np.empty((1, len(items)), dtype=object)
    for k, x in enumerate(items):
        c[0, k] = x
    return c


def save_data(path: str, data, profile: dict):
    """``save data_MNAD_Acoustic data profile`` (main_Acoustic_RTM.m:183,
    main_Acoustic_Data.m:179): ``data`` is the 1 x ns cell of the forward's
    returns, each the 1 x 1 cell ``{datau}``; pass the per-shot ``datau``
    (nt x nr) arrays or the one-element lists ``fwd_PDE_exact_MNAD`` returns."""
    shots = [d[0] if isinstance(d, (list, tuple)) else d for d in data]
    _savemat(path, {"data": _cell_row([_cell_row([np.asarray(d, dtype=np.float64)]) for d in shots]),
                    "profile": {k: profile[k] for k in PROFILE_FIELDS}})


def save_scattered(path: str, data_sct, profile: dict):
    """``save data_scattered_MNAD_Acoustic data_sct profile``
    (main_Acoustic_RTM.m:234): the 1 x ns cell of scattered gathers."""
    _savemat(path, {"data_sct": _cell_row([np.asarray(d, dtype=np.float64) for d in data_sct]),
                    "profile": {k: profile[k] for k in PROFILE_FIELDS}})


def load_data(path: str):
    """(per-shot ``datau`` arrays, profile dict) of a file written by
    :func:`save_data` or by the reference driver."""
    import scipy.io
    m = scipy.io.loadmat(path)
    cells = m["data"]
    shots = [np.asarray(cells[0, k][0, 0]) for k in range(cells.shape[1])]
    prof = m["profile"][0, 0]
    return shots, {k: float(prof[k][0, 0]) for k in prof.dtype.names}


def save_illum_average(path: str, illum):
    """``save(['./Illuminations/illum_' num2str(0)],'illum')``
    (main_Acoustic_RTM.m:237-244): the illumination averaged over the shots."""
    _savemat(path, {"illum": np.asarray(illum, dtype=np.float64)})
