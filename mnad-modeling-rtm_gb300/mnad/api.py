"""Python front end of the MNAD GB300 library (contexts, shots, batched plans).

Arrays follow the reference's MATLAB conventions: models are ``(nz, nx)``
padded grids (z = rows), receiver data is ``(nt, nr)``, images and
illumination are returned as ``(nz-2*d_pml, nx-2*d_pml)`` arrays (the
reference's ``Nint x 1`` vectors reshaped column-major).  Indices are 1-based.
All compute runs in libmnad.so on the GPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import Job, MnadError, Options, check, lib

_CODECS = {"f32": _lib.SNAP_F32, "bf16": _lib.SNAP_BF16, "f16": _lib.SNAP_F16}
_PAIRINGS = {"reference": _lib.PAIR_REFERENCE, "aligned": _lib.PAIR_ALIGNED}
_KERNELS = {"auto": _lib.KERNEL_AUTO, "direct": _lib.KERNEL_DIRECT, "tma": _lib.KERNEL_TMA,
            "tune": _lib.KERNEL_TUNE, "tma2": _lib.KERNEL_TMA2, "tma_narrow": _lib.KERNEL_TMA_NARROW}


def _f64(a, order="F"):
    return np.require(np.asarray(a, dtype=np.float64), requirements=[order[0], "A"])


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _vec(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())


class Context:
    """One CUDA context/stream on one GPU plus its stored source wavefields."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, **options):
        h = C.c_void_p()
        check(lib().mnad_context_create(device, hbm_budget, C.byref(h)))
        self._h = h
        if options:
            self.set_options(**options)

    def close(self):
        if getattr(self, "_h", None):
            check(lib().mnad_context_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- options -----------------------------------------------------------
    def options(self) -> dict:
        o = Options()
        check(lib().mnad_context_get_options(self._h, C.byref(o)))
        inv = lambda d, v: next(k for k, x in d.items() if x == v)
        return {"snapshot_codec": inv(_CODECS, o.snapshot_codec), "pairing": inv(_PAIRINGS, o.pairing),
                "T": o.T, "record_vw": bool(o.record_vw), "use_graphs": bool(o.use_graphs),
                "kernel": inv(_KERNELS, o.kernel), "energy_every": o.energy_every,
                "checkpoint_every": o.checkpoint_every, "checkpoint_codec": inv(_CODECS, o.checkpoint_codec)}

    def set_options(self, snapshot_codec=None, pairing=None, T=None, record_vw=None, use_graphs=None,
                    kernel=None, energy_every=None, checkpoint_every=None, checkpoint_codec=None):
        o = Options()
        check(lib().mnad_context_get_options(self._h, C.byref(o)))
        if snapshot_codec is not None:
            o.snapshot_codec = _CODECS[snapshot_codec]
        if pairing is not None:
            o.pairing = _PAIRINGS[pairing]
        if T is not None:
            o.T = int(T)
        if record_vw is not None:
            o.record_vw = int(bool(record_vw))
        if use_graphs is not None:
            o.use_graphs = int(bool(use_graphs))
        if kernel is not None:
            o.kernel = _KERNELS[kernel]
        if energy_every is not None:
            o.energy_every = int(energy_every)
        if checkpoint_every is not None:
            o.checkpoint_every = int(checkpoint_every)
        if checkpoint_codec is not None:
            o.checkpoint_codec = _CODECS[checkpoint_codec]
        check(lib().mnad_context_set_options(self._h, C.byref(o)))

    def memory(self) -> int:
        n = C.c_size_t()
        check(lib().mnad_context_memory(self._h, C.byref(n)))
        return n.value

    def transfers(self):
        """(h2d_bytes, d2h_bytes) copied by this context so far."""
        a, b = C.c_uint64(), C.c_uint64()
        check(lib().mnad_context_transfers(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def energy(self) -> np.ndarray:
        """Energy history of the last forward (see mnad_context_energy)."""
        n = C.c_int()
        check(lib().mnad_context_energy(self._h, None, 0, C.byref(n)))
        out = np.zeros(n.value)
        check(lib().mnad_context_energy(self._h, _ptr(out), n.value, C.byref(n)))
        return out

    def status(self) -> int:
        f = C.c_uint()
        check(lib().mnad_context_status(self._h, C.byref(f)))
        return f.value

    def set_wait_limit(self, polls: int = 0):
        """Bound of the step kernel's barrier waits (0: default); see mnad_context_set_wait_limit."""
        check(lib().mnad_context_set_wait_limit(self._h, int(polls)))

    # -- drop-in shots -----------------------------------------------------
    def fwd(self, dx, xs, xr, dz, zs, zr, v, dt, nt, w, d_pml, ss=1, indx=0, record_vw=False):
        """fwd_PDE_exact_MNAD on the GPU; returns datau (nt, nr) or (datau, datav, dataw)."""
        v = _f64(v)
        nz, nx = v.shape
        xr, zr, w = _vec(xr), _vec(zr), _vec(w)
        if xr.size != zr.size:
            raise MnadError(_lib.E_ARG, "xr and zr differ in length")
        nr = xr.size
        if w.size < nt:
            raise MnadError(_lib.E_ARG, f"w has {w.size} samples, nt = {nt}")
        datau = np.zeros((nt, nr), order="F")
        datav = np.zeros((nt, nr), order="F") if record_vw else None
        dataw = np.zeros((nt, nr), order="F") if record_vw else None
        if record_vw:
            self.set_options(record_vw=True)
        try:
            check(lib().mnad_fwd_pde_exact(self._h, float(dx), float(xs), _ptr(xr), nr, float(dz), float(zs),
                                           _ptr(zr), _ptr(v), nz, nx, float(dt), int(nt), _ptr(w), int(d_pml),
                                           int(ss), int(indx), _ptr(datau), _ptr(datav), _ptr(dataw)))
        finally:
            if record_vw:
                self.set_options(record_vw=False)
        return (datau, datav, dataw) if record_vw else datau

    def fwd_fields(self, dx, xs, xr, dz, zs, zr, v, dt, nt, w, d_pml, steps):
        """Forward shot that also returns {tt: (nU, nV, nW)} after each listed step."""
        v = _f64(v)
        nz, nx = v.shape
        xr, zr, w = _vec(xr), _vec(zr), _vec(w)
        nr = xr.size
        steps = np.ascontiguousarray(np.asarray(steps, dtype=np.int32).ravel())
        datau = np.zeros((nt, nr), order="F")
        fields = np.zeros(max(1, steps.size) * 3 * nz * nx)
        check(lib().mnad_fwd_fields(self._h, float(dx), float(xs), _ptr(xr), nr, float(dz), float(zs), _ptr(zr),
                                    _ptr(v), nz, nx, float(dt), int(nt), _ptr(w), int(d_pml), steps.size,
                                    steps.ctypes.data_as(C.POINTER(C.c_int)), _ptr(datau), _ptr(fields)))
        n = nz * nx
        out = {int(t): tuple(fields[(k * 3 + f) * n:(k * 3 + f + 1) * n].reshape((nz, nx), order="F")
                             for f in range(3)) for k, t in enumerate(steps)}
        return datau, out

    def adj(self, dx, dz, nt, dt, v, xr, zr, data, d_pml, ss=1):
        """Born_adj_MNAD on the GPU; returns the image, shape (nz-2d, nx-2d), times T."""
        v = _f64(v)
        nz, nx = v.shape
        if isinstance(data, (list, tuple)):
            data = data[0]
        data = _f64(data)
        xr, zr = _vec(xr), _vec(zr)
        nr = xr.size
        if data.shape != (nt, nr):
            raise MnadError(_lib.E_ARG, f"data must be (nt, nr) = ({nt}, {nr}), got {data.shape}")
        im = np.zeros((nz - 2 * d_pml, nx - 2 * d_pml), order="F")
        check(lib().mnad_born_adj(self._h, float(dx), float(dz), int(nt), float(dt), _ptr(v), nz, nx, _ptr(xr),
                                  _ptr(zr), nr, _ptr(data), int(d_pml), int(ss), _ptr(im)))
        return im

    # -- stored wavefields ---------------------------------------------------
    def wavefield_info(self, ss):
        nint, ncols, nsnap, T = C.c_int64(), C.c_int(), C.c_int(), C.c_int()
        check(lib().mnad_wavefield_info(self._h, int(ss), C.byref(nint), C.byref(ncols), C.byref(nsnap),
                                        C.byref(T)))
        return {"nint": nint.value, "ncols": ncols.value, "nsnap": nsnap.value, "T": T.value}

    def wavefield_export(self, ss, shape_int=None):
        """(UU, illum) as the reference saves them (UU: Nint x ncols, illum: T*sum d2u^2)."""
        info = self.wavefield_info(ss)
        UU = np.zeros((info["nint"], info["ncols"]), order="F")
        illum = np.zeros(info["nint"])
        check(lib().mnad_wavefield_export(self._h, int(ss), _ptr(UU), _ptr(illum)))
        if shape_int is not None:
            illum = illum.reshape(shape_int, order="F")
        return UU, illum

    def wavefield_import(self, ss, nz, nx, d_pml, nt, T, UU, nsnap=None, illum=None):
        UU = _f64(UU)
        nint, ncols = UU.shape
        nsnap = ncols if nsnap is None else int(nsnap)
        il = None if illum is None else _vec(illum)
        check(lib().mnad_wavefield_import(self._h, int(ss), nz, nx, d_pml, int(nt), int(T), ncols, nsnap,
                                          _ptr(UU), _ptr(il)))

    def wavefield_release(self, ss):
        check(lib().mnad_wavefield_release(self._h, int(ss)))

    # -- batched jobs ----------------------------------------------------------
    def plan(self, jobs: Sequence["ShotJob"]) -> "Plan":
        return Plan(self, jobs)

    def run_jobs(self, jobs: Sequence["ShotJob"]):
        arr, keep = _job_array(jobs)
        check(lib().mnad_run_jobs(self._h, arr, len(jobs)))
        return jobs


@dataclass
class ShotJob:
    """One modeling (kind='model') or RTM (kind='rtm') shot of a batch.

    Outputs are allocated here: ``data`` (nt, nr) (model: gather; rtm:
    scattered data), ``image`` and ``illum`` (nz-2d, nx-2d) for RTM.
    """
    kind: str
    v: np.ndarray
    dx: float
    dz: float
    dt: float
    nt: int
    d_pml: int
    zs: float
    xs: float
    zr: np.ndarray
    xr: np.ndarray
    w: np.ndarray
    vs: Optional[np.ndarray] = None
    T: int = 0
    keep_data: bool = True
    data: Optional[np.ndarray] = None
    image: Optional[np.ndarray] = None
    illum: Optional[np.ndarray] = None

    def __post_init__(self):
        self.v = _f64(self.v)
        if self.vs is not None:
            self.vs = _f64(self.vs)
        self.zr, self.xr, self.w = _vec(self.zr), _vec(self.xr), _vec(self.w)
        nz, nx = self.v.shape
        nr = self.xr.size
        if self.kind == "model" or self.keep_data:
            self.data = np.zeros((self.nt, nr), order="F")
        if self.kind == "rtm":
            self.image = np.zeros((nz - 2 * self.d_pml, nx - 2 * self.d_pml), order="F")
            self.illum = np.zeros_like(self.image)


def _job_array(jobs):
    arr = (Job * max(1, len(jobs)))()
    keep = []
    for k, j in enumerate(jobs):
        nz, nx = j.v.shape
        J = arr[k]
        J.kind = _lib.JOB_RTM if j.kind == "rtm" else _lib.JOB_MODEL
        J.nz, J.nx, J.d_pml, J.nt = nz, nx, int(j.d_pml), int(j.nt)
        J.dx, J.dz, J.dt = float(j.dx), float(j.dz), float(j.dt)
        J.v, J.vs = _ptr(j.v), _ptr(j.vs)
        J.zs, J.xs = float(j.zs), float(j.xs)
        J.nr = j.xr.size
        J.zr, J.xr, J.w = _ptr(j.zr), _ptr(j.xr), _ptr(j.w)
        J.T = int(j.T)
        J.data_out = _ptr(j.data)
        J.image_out = _ptr(j.image)
        J.illum_out = _ptr(j.illum)
        keep.append(j)
    return arr, keep


class Plan:
    """Device-resident batch: inputs uploaded once, ``run()`` repeatable."""

    def __init__(self, ctx: Context, jobs: Sequence[ShotJob]):
        self.ctx = ctx
        self.jobs = list(jobs)
        self._arr, self._keep = _job_array(self.jobs)
        h = C.c_void_p()
        check(lib().mnad_plan_create(ctx.handle, self._arr, len(self.jobs), C.byref(h)))
        self._h = h

    def run(self):
        check(lib().mnad_plan_run(self._h))

    def download(self):
        check(lib().mnad_plan_download(self._h))
        return self.jobs

    def work(self):
        p, b = C.c_double(), C.c_double()
        check(lib().mnad_plan_work(self._h, C.byref(p), C.byref(b)))
        return p.value, b.value

    def timing(self):
        r, s, n = C.c_double(), C.c_double(), C.c_int()
        check(lib().mnad_plan_timing(self._h, C.byref(r), C.byref(s), C.byref(n)))
        return {"run_ms": r.value, "step_ms": s.value, "step_launches": n.value}

    def phases(self):
        """Device time (ms) and algorithmic bytes of the last run's forward
        phase and adjoint phase."""
        v = [C.c_double() for _ in range(4)]
        check(lib().mnad_plan_phases(self._h, *[C.byref(x) for x in v]))
        return {"forward_ms": v[0].value, "forward_bytes": v[1].value, "adjoint_ms": v[2].value,
                "adjoint_bytes": v[3].value}

    def kernels(self):
        """{'forward': name, 'adjoint': name} of the step kernels the phases run
        (the largest launch group of each; None where a phase is empty)."""
        f, a = C.c_int(), C.c_int()
        check(lib().mnad_plan_kernels(self._h, C.byref(f), C.byref(a)))
        names = {v: k for k, v in _KERNELS.items()}
        return {"forward": names.get(f.value), "adjoint": names.get(a.value)}

    def stack(self):
        """(image_sum, illum_sum, img_rtm) of the RTM shots, (nz-2d, nx-2d) arrays."""
        rtm = [j for j in self.jobs if j.kind == "rtm"]
        if not rtm:
            raise MnadError(_lib.E_ARG, "the plan has no RTM job")
        shape = rtm[0].image.shape
        outs = [np.zeros(shape, order="F") for _ in range(3)]
        check(lib().mnad_plan_stack(self._h, *[_ptr(o) for o in outs]))
        return tuple(outs)

    def close(self):
        if getattr(self, "_h", None):
            check(lib().mnad_plan_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching server on one device (``mnad_server_*``).

    ``submit`` copies a :class:`ShotJob`'s inputs and queues it; the worker
    writes the outputs into the job's arrays, which this object keeps alive
    until ``wait`` has seen the job finish.
    """

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, chunk_steps: int = 64, max_active_jobs: int = 0,
                 snapshot_codec: str = "f32", kernel: str = "auto", graphs: bool = True):
        o = _lib.ServerOptions()
        o.no_graphs = 0 if graphs else 1
        o.hbm_budget_bytes = int(hbm_budget_bytes)
        o.chunk_steps = int(chunk_steps)
        o.max_active_jobs = int(max_active_jobs)
        o.snapshot_codec = _CODECS[snapshot_codec]
        o.kernel = _KERNELS[kernel]
        h = C.c_void_p()
        check(lib().mnad_server_create(int(device), C.byref(o), C.byref(h)))
        self._h = h
        self._jobs = {}

    def submit(self, job: ShotJob) -> int:
        arr, _ = _job_array([job])
        t = C.c_uint64()
        check(lib().mnad_server_submit(self._h, arr, C.byref(t)))
        self._jobs[t.value] = job
        return t.value

    def poll(self, ticket: int) -> str:
        s = C.c_int()
        check(lib().mnad_server_poll(self._h, int(ticket), C.byref(s)))
        return ("queued", "running", "done", "failed")[s.value]

    def wait(self, ticket: int, timeout_s: float = -1.0) -> ShotJob:
        """Block until the job is done and return it (raises its error)."""
        rc = lib().mnad_server_wait(self._h, int(ticket), float(timeout_s))
        if rc != _lib.E_TIMEOUT:
            job = self._jobs.pop(int(ticket), None)
        check(rc)
        return job

    def stats(self) -> dict:
        s = _lib.ServerStats()
        check(lib().mnad_server_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in _lib.ServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            check(lib().mnad_server_destroy(self._h))
            self._h = None
            self._jobs.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
