"""The reference's two driver scripts as functions on the GPU library.

``acoustic_rtm`` follows ``SRC/migration/main_Acoustic_RTM.m``:
  1. grid and time rules (dx from the minimum wavelength, dt from the CFL
     rule, t = 0:dt:T_max-dt), lines 70-90;
  2. the acquisition (``acquisi``), padded indices, lines 120-130;
  3. the Ricker wavelet, lines 138-140;
  4. edge-replicated padding, lines 148-149;
  5. the migration model ``v_smooth(V, sindx, sindx, sindx)``, lines 195-197;
  6. per shot: true-model forward, background forward with snapshots,
     scattered data, adjoint with imaging -- the two ``parfor`` loops, here
     one batched plan on the GPU;
  7. ``img_RTM = mean(mhh,3) ./ illum``, lines 237-262 (FP64 on the device).

``acoustic_data`` follows ``SRC/modeling/main_Acoustic_Data.m`` (the same
rules and acquisition, forward modeling only).

The nine sparse operators the scripts assemble are not built: the library
recomputes the same coefficients on the device.
"""
from __future__ import annotations

import math
from typing import Optional

import numpy as np

from . import workflow
from .api import Context, ShotJob


def grid_and_time(V, fc: float, T_max: float):
    """(dx, dz, dt, nt) of the drivers: f_max = 3 fc, dx = dz =
    floor(Vmin / (2.5 f_max)), dt = 0.8 * 0.65 * (unrounded dx) / Vmax,
    nt = length(0:dt:T_max-dt)."""
    V = np.asarray(V, dtype=np.float64)
    vmin, vmax = float(V.min()), float(V.max())
    f_max = 3.0 * fc
    dx = vmin / (2.5 * f_max)
    dt = 0.8 * ((0.65 * dx) / vmax)
    nt = int(math.floor((T_max - dt) / dt * (1 + 1e-15) + 1e-10)) + 1
    return float(math.floor(dx)), float(math.floor(dx)), dt, nt


def _geometry(V, dx, dz, d_pml, acq):
    Source, Receiver = workflow.acquisi(V, dx, dz, **acq)
    xs, zs, xr, zr = workflow.padded_indices(Source, Receiver, dx, dz, d_pml)
    return Source, Receiver, xs, zs, xr, zr


def _default_acq(dx, dz, zsc=2, zrc=4, h_offset=1, ds=10, dr=1, slag=1, rlag=1, acq_type="fixspread"):
    return dict(zsc=zsc * dz, zrc=zrc * dz, h_offset=h_offset * dx, ds=ds * dx, dr=dr * dx, slag=slag * dx,
                rlag=rlag * dx, acq_type=acq_type)


def acoustic_rtm(V, fc: float = 15.0, T_max: float = 3.0, d_pml: int = 40, sindx: int = 3,
                 acquisition: Optional[dict] = None, ctx: Optional[Context] = None, **ctx_options):
    """RTM of every shot of the acquisition over the physical model ``V``
    (nz x nx); returns a dict with ``img_RTM`` (nz x nx), ``image_sum``,
    ``illum`` (mean illumination), ``data_sct`` (scattered data per shot) and
    ``profile`` (the scripts' parameters).  ``acquisition`` holds the
    geometry of ``acquisi`` in grid units of dx / dz (the script's defaults:
    zsc 2, zrc 4, h_offset 1, ds 10, dr 1, slag 1, rlag 1, 'fixspread')."""
    V = np.asarray(V, dtype=np.float64)
    dx, dz, dt, nt = grid_and_time(V, fc, T_max)
    acq = _default_acq(dx, dz, **(acquisition or {}))
    Source, Receiver, xs, zs, xr, zr = _geometry(V, dx, dz, d_pml, acq)
    w = workflow.ricker(fc, dt, nt)
    v = np.asfortranarray(workflow.pad_model(V, d_pml))
    vs = np.asfortranarray(workflow.pad_model(workflow.v_smooth(V, sindx, sindx, sindx), d_pml))
    jobs = [ShotJob(kind="rtm", v=v, vs=vs, dx=dx, dz=dz, dt=dt, nt=nt, d_pml=d_pml, zs=float(zs[k]),
                    xs=float(xs[k]), zr=zr[k], xr=xr[k], w=w, keep_data=True) for k in range(len(xs))]
    own = ctx is None
    ctx = ctx or Context(0, **ctx_options)
    try:
        plan = ctx.plan(jobs)
        plan.run()
        plan.download()
        image_sum, illum_sum, img = plan.stack()
        plan.close()
    finally:
        if own:
            ctx.close()
    ns = len(jobs)
    profile = dict(fc=fc, f_max=3 * fc, dt=dt, T_max=T_max, nt=nt, dx=dx, dz=dz, nx=V.shape[1], nz=V.shape[0],
                   ns=ns, Source=Source, Receiver=Receiver, w=w, d_pml=d_pml)
    return dict(img_RTM=img, image_sum=image_sum, illum=illum_sum / ns, data_sct=[j.data for j in jobs],
                profile=profile)


def acoustic_data(V, fc: float = 10.0, T_max: float = 3.0, d_pml: int = 40, acquisition: Optional[dict] = None,
                  ctx: Optional[Context] = None, **ctx_options):
    """Forward modeling of every shot (``main_Acoustic_Data.m``); returns
    ``(data, profile)`` with one nt x nr gather per shot."""
    V = np.asarray(V, dtype=np.float64)
    dx, dz, dt, nt = grid_and_time(V, fc, T_max)
    acq = _default_acq(dx, dz, **(acquisition or {}))
    Source, Receiver, xs, zs, xr, zr = _geometry(V, dx, dz, d_pml, acq)
    w = workflow.ricker(fc, dt, nt)
    v = np.asfortranarray(workflow.pad_model(V, d_pml))
    jobs = [ShotJob(kind="model", v=v, dx=dx, dz=dz, dt=dt, nt=nt, d_pml=d_pml, zs=float(zs[k]), xs=float(xs[k]),
                    zr=zr[k], xr=xr[k], w=w) for k in range(len(xs))]
    own = ctx is None
    ctx = ctx or Context(0, **ctx_options)
    try:
        ctx.run_jobs(jobs)
    finally:
        if own:
            ctx.close()
    profile = dict(fc=fc, f_max=3 * fc, dt=dt, T_max=T_max, nt=nt, dx=dx, dz=dz, nx=V.shape[1], nz=V.shape[0],
                   ns=len(jobs), Source=Source, Receiver=Receiver, w=w, d_pml=d_pml)
    return [j.data for j in jobs], profile
