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
    import scipy.io
    UU, illum = ctx.wavefield_export(ss)
    os.makedirs(os.path.join(directory, "Wavefields"), exist_ok=True)
    os.makedirs(os.path.join(directory, "Illuminations"), exist_ok=True)
    scipy.io.savemat(os.path.join(directory, "Wavefields", f"UU_{ss}.mat"), {"UU": UU})
    scipy.io.savemat(os.path.join(directory, "Illuminations", f"illum_{ss}.mat"),
                     {"illum": illum.reshape((nz - 2 * d_pml, nx - 2 * d_pml), order="F")})


def load_wavefield(ctx: Context, ss: int, nz: int, nx: int, d_pml: int, nt: int, T: int, directory: str = "."):
    """Read ``Wavefields/UU_<ss>.mat`` back into device storage for shot ``ss``
    (the ``load`` at ``Born_adj_MNAD.m:33``).  Trailing all-zero columns of
    the reference's preallocated matrix stay part of ``ncols``."""
    import scipy.io
    UU = scipy.io.loadmat(os.path.join(directory, "Wavefields", f"UU_{ss}.mat"))["UU"]
    nsnap = nt // T
    ctx.wavefield_import(ss, nz, nx, d_pml, nt, T, UU, nsnap=min(nsnap, UU.shape[1]))
