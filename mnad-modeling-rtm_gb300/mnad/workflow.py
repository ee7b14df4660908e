"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset is involved: every model is generated here from a seed.  The
drivers' conventions are kept: the physical model is padded by edge
replication (``SRC/migration/main_Acoustic_RTM.m:148-149``), the Ricker
wavelet is ``(1-2 tau^2) exp(-tau^2)``, ``tau = pi (t - 1.1/fc) fc``
(``:138-140``), and grid indices are ``d_pml + metres/dx`` with
``metres = dx * grid index`` (``:124-130`` with ``SRC/MNAD/acquisi.m:122-123,
194``).  Receivers and sources are given as 1-based padded indices.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np


def ricker(fc: float, dt: float, nt: int) -> np.ndarray:
    t = np.arange(nt) * dt
    tau = np.pi * (t - 1.1 / fc) * fc
    return (1 - 2 * tau**2) * np.exp(-tau**2)


def pad_model(V: np.ndarray, d: int) -> np.ndarray:
    V = np.asarray(V, dtype=np.float64)
    return np.pad(V, ((d, d), (d, d)), mode="edge")


def gaussian_smooth(V: np.ndarray, taps: int, sigma: Optional[float] = None) -> np.ndarray:
    """Separable Gaussian of ``taps`` points (sigma = taps/6 by default), edge-replicated."""
    sigma = taps / 6.0 if sigma is None else sigma
    h = taps // 2
    k = np.exp(-0.5 * (np.arange(-h, h + 1) / sigma) ** 2)
    k /= k.sum()
    out = np.asarray(V, dtype=np.float64)
    for ax in (0, 1):
        p = np.pad(out, [(h, h) if a == ax else (0, 0) for a in (0, 1)], mode="edge")
        acc = np.zeros_like(out)
        for t in range(taps):
            sl = [slice(None), slice(None)]
            sl[ax] = slice(t, t + out.shape[ax])
            acc += k[t] * p[tuple(sl)]
        out = acc
    return out


@dataclass
class Shot:
    zs: int
    xs: int
    zr: np.ndarray
    xr: np.ndarray


@dataclass
class Survey:
    """A padded model (true and optionally migration), grid, time axis, shots."""
    name: str
    v: np.ndarray                     # padded true model (nz, nx)
    dx: float
    dz: float
    dt: float
    nt: int
    d_pml: int
    fc: float
    shots: List[Shot]
    vs: Optional[np.ndarray] = None   # padded migration model
    T: int = 0                        # snapshot interval (0: reference formula)
    codec: str = "f32"
    meta: dict = field(default_factory=dict)

    @property
    def w(self) -> np.ndarray:
        return ricker(self.fc, self.dt, self.nt)

    @property
    def nz(self):
        return self.v.shape[0]

    @property
    def nx(self):
        return self.v.shape[1]


def constant_velocity_shot(nt: int = 1000) -> Survey:
    """Plain FP64 forward modeling: 201 x 201 total grid (physical 161 x 161
    plus a 20-point CPML), 10 m, 2000 m/s, 20 Hz Ricker at (101,101),
    dt = 1 ms, 201 receivers on row 21 (the first physical row)."""
    d = 20
    v = np.full((201, 201), 2000.0)
    shot = Shot(101, 101, np.full(201, 21), np.arange(1, 202))
    return Survey("constant velocity 201x201", v, 10.0, 10.0, 1e-3, nt, d, 20.0, [shot])


def layered_anomaly_shot(seed: int = 0, nt: int = 3000, T: int = 4) -> Survey:
    """Single-shot RTM: 301 (z) x 601 (x) at 10 m, layers 1500/2000/2600/3200
    m/s with interfaces at 800/1600/2400 m, +300 m/s Gaussian anomaly
    (sigma 150 m, centre from the seed); migration model = true model
    smoothed by a 15-point Gaussian; 15 Hz; shot at x = 3000 m; 601
    receivers at z = 20 m; dt = 1 ms; 3 s; snapshots every T = 4 steps."""
    rng = np.random.default_rng(seed)
    nzp, nxp, h, d = 301, 601, 10.0, 40
    z = np.arange(nzp)[:, None] * h
    x = np.arange(nxp)[None, :] * h
    V = np.where(z < 800, 1500.0, np.where(z < 1600, 2000.0, np.where(z < 2400, 2600.0, 3200.0)))
    V = np.broadcast_to(V, (nzp, nxp)).copy()
    cz = rng.uniform(900, 2200)
    cx = rng.uniform(1500, 4500)
    V += 300.0 * np.exp(-((z - cz) ** 2 + (x - cx) ** 2) / (2 * 150.0**2))
    Vs = gaussian_smooth(V, 15)
    xs_grid, zs_grid, zr_grid = 300, 1, 2
    shot = Shot(d + zs_grid, d + xs_grid, np.full(nxp, d + zr_grid), d + np.arange(1, nxp + 1))
    return Survey("layered + anomaly 301x601", pad_model(V, d), h, h, 1e-3, nt, d, 15.0, [shot], vs=pad_model(Vs, d), T=T,
                  meta={"anomaly_centre_m": (cz, cx)})


def gaussian_random_field(shape, h, corr, rng):
    """Unit-variance field with a Gaussian covariance of correlation length ``corr`` (m)."""
    nz, nx = shape
    kz = np.fft.fftfreq(nz, d=h)[:, None]
    kx = np.fft.fftfreq(nx, d=h)[None, :]
    spec = np.exp(-((np.pi * corr) ** 2) * (kz**2 + kx**2) / 2)
    f = np.real(np.fft.ifft2(np.fft.fft2(rng.standard_normal(shape)) * spec))
    return (f - f.mean()) / (f.std() + 1e-30)


def random_field_survey(seed: int = 0, nshots: int = 64, nt: int = 4000, codec: str = "bf16") -> Survey:
    """Batched RTM: 401 (z) x 1201 (x) at 12.5 m; smooth Gaussian random field
    (correlation 300 m) clipped to 1500-4000 m/s plus three dipping
    +400 m/s reflectors; ``nshots`` shots every 187.5 m; 20 Hz; dt = 1 ms;
    4 s; BF16 snapshots; migration model = 15-point Gaussian smoothing."""
    rng = np.random.default_rng(seed)
    nzp, nxp, h, d = 401, 1201, 12.5, 40
    g = gaussian_random_field((nzp, nxp), h, 300.0, rng)
    V = np.clip(2750.0 + 600.0 * g, 1500.0, 4000.0)
    z = np.arange(nzp)[:, None] * h
    x = np.arange(nxp)[None, :] * h
    for _ in range(3):
        z0 = rng.uniform(1200, 4200)
        dip = np.tan(np.deg2rad(rng.uniform(-12, 12)))
        band = np.abs(z - (z0 + dip * (x - x.mean()))) < 1.5 * h
        V = V + 400.0 * band
    Vs = gaussian_smooth(V, 15)
    # 187.5 m apart; a longer shot list (shards of a multi-GPU run) is spread
    # evenly over the line instead
    spacing = max(1, min(int(round(187.5 / h)), (nxp - 1) // max(nshots, 1)))
    first = (nxp - spacing * (nshots - 1)) // 2
    shots = []
    for s in range(nshots):
        xg = max(1, min(nxp, first + s * spacing))
        shots.append(Shot(d + 1, d + xg, np.full(nxp, d + 2), d + np.arange(1, nxp + 1)))
    return Survey("random field 401x1201", pad_model(V, d), h, h, 1e-3, nt, d, 20.0, shots, vs=pad_model(Vs, d), codec=codec)


def faulted_model(nz: int, nx: int, h: float, rng, nfaults: int = 6) -> np.ndarray:
    """Seeded faulted sedimentary model: 10-16 layers whose velocities rise
    with depth from 1500 to about 4000 m/s (gently undulating interfaces; the
    first at 2-4 % of the depth, the others within the upper 60 %, so that a
    record of a few seconds sees reflections), ``nfaults`` normal faults
    (60-70 degree dip, 40-200 m throw, hanging wall down) and a salt-like
    4500 m/s body at 30-45 % of the depth; clipped to 1500-4500 m/s."""
    z = np.arange(nz, dtype=np.float64)[:, None] * h
    x = np.arange(nx, dtype=np.float64)[None, :] * h
    zmax, xmax = nz * h, nx * h
    # depth in the layer frame: faults shift the hanging wall down by the throw
    zl = np.broadcast_to(z, (nz, nx)).copy()
    for _ in range(nfaults):
        x0 = rng.uniform(0.1, 0.9) * xmax
        dip = np.deg2rad(rng.uniform(60.0, 70.0)) * rng.choice((-1.0, 1.0))
        throw = rng.uniform(40.0, 200.0)
        hanging = (x - x0) * np.sign(dip) > (z / np.tan(abs(dip)))
        zl -= throw * hanging
    nl = int(rng.integers(10, 17))
    tops = np.sort(np.concatenate(([rng.uniform(0.02, 0.04)], rng.uniform(0.04, 0.6, nl - 2)))) * zmax
    vel = np.sort(rng.uniform(1500.0, 4000.0, nl))
    vel[0] = 1500.0
    und = 0.01 * zmax * np.sin(2 * np.pi * x / rng.uniform(0.2, 0.6) / xmax + rng.uniform(0, 2 * np.pi))
    V = vel[np.searchsorted(tops, zl + und, side="right")]
    # salt body: an ellipse with a rough top
    cz, cx = rng.uniform(0.3, 0.45) * zmax, rng.uniform(0.3, 0.7) * xmax
    az, ax = rng.uniform(0.08, 0.15) * zmax, rng.uniform(0.06, 0.12) * xmax
    rough = 1.0 + 0.15 * np.sin(5 * np.pi * x / xmax + rng.uniform(0, 2 * np.pi))
    V = np.where(((z - cz) / (az * rough)) ** 2 + ((x - cx) / ax) ** 2 < 1.0, 4500.0, V)
    return np.clip(V, 1500.0, 4500.0)


def faulted_salt_survey(seed: int = 0, nshots: int = 256, nt: int = 6000, first: int = 0, count: Optional[int] = None) -> Survey:
    """Large-scale RTM at 2 points per minimum wavelength: 1201 (z) x 4001 (x)
    at 12.5 m (1281 x 4081 padded), vmin 1500 m/s; seeded faulted
    sedimentary model with a 4500 m/s salt body; ``nshots`` shots spread over
    the line, receivers on every column at 25 m depth; 25 Hz Ricker; dt =
    1 ms; 6 s; migration model = 15-point Gaussian smoothing.  ``first`` /
    ``count`` select a subset of the shots (same model)."""
    rng = np.random.default_rng(seed)
    nzp, nxp, h, d = 1201, 4001, 12.5, 40
    V = faulted_model(nzp, nxp, h, rng)
    Vs = gaussian_smooth(V, 15)
    step = (nxp - 1) / max(nshots, 1)
    count = nshots - first if count is None else count
    shots = []
    for s in range(first, first + count):
        xg = int(round(step * (s + 0.5))) + 1
        shots.append(Shot(d + 1, d + xg, np.full(nxp, d + 2), d + np.arange(1, nxp + 1)))
    return Survey("faulted + salt 1201x4001", pad_model(V, d), h, h, 1e-3, nt, d, 25.0, shots, vs=pad_model(Vs, d), codec="f32",
                  meta={"nshots_total": nshots})


def shot_jobs(sv: Survey, kind: str = "rtm", shots=None, keep_data: bool = False):
    """mnad.api.ShotJob list for a survey (RTM: true + migration model)."""
    from .api import ShotJob
    # one column-major copy of each model shared by every job: the library
    # uploads a model array once per plan however many shots use it
    v = np.asfortranarray(sv.v, dtype=np.float64)
    vs = np.asfortranarray(sv.vs, dtype=np.float64) if (kind == "rtm" and sv.vs is not None) else None
    w = sv.w
    out = []
    for sh in (sv.shots if shots is None else shots):
        out.append(ShotJob(kind=kind, v=v, vs=vs, dx=sv.dx, dz=sv.dz, dt=sv.dt,
                           nt=sv.nt, d_pml=sv.d_pml, zs=sh.zs, xs=sh.xs, zr=sh.zr, xr=sh.xr, w=w, T=sv.T,
                           keep_data=keep_data))
    return out


# Served shot stream: grids (nz, nx) of the total (CPML-padded) model.
SERVED_GRIDS = ((256, 256), (256, 512), (512, 1024), (1024, 2048))
SERVED_SECONDS = (1.0, 2.0, 4.0)


def layered_anomaly_model(nz: int, nx: int, h: float, rng) -> np.ndarray:
    """Random layered model (3-6 layers, increasing with depth, 1500-4500 m/s)
    with a Gaussian anomaly of +-(150-400) m/s, clipped to 1500-4500 m/s."""
    nl = int(rng.integers(3, 7))
    tops = np.sort(rng.uniform(0.1, 0.9, nl - 1)) * nz
    vel = np.sort(rng.uniform(1500.0, 4500.0, nl))
    z = np.arange(nz, dtype=np.float64)[:, None]
    x = np.arange(nx, dtype=np.float64)[None, :]
    layer = np.searchsorted(tops, z, side="right") * np.ones((1, nx), dtype=np.int64)
    V = vel[layer]
    cz, cx = rng.uniform(0.2, 0.8) * nz, rng.uniform(0.2, 0.8) * nx
    sig = rng.uniform(100.0, 300.0) / h
    amp = rng.uniform(150.0, 400.0) * rng.choice((-1.0, 1.0))
    V = V + amp * np.exp(-((z - cz) ** 2 + (x - cx) ** 2) / (2 * sig ** 2))
    return np.clip(V, 1500.0, 4500.0)


@dataclass
class ServedJob:
    arrival_s: float
    kind: str
    grid: tuple
    nt: int
    fc: float
    model: int        # index into the stream's model pool of that grid
    xs: int           # 1-based padded source column


def served_stream(seed: int = 0, njobs: int = 512, rate: Optional[float] = None, models_per_grid: int = 4,
            d_pml: int = 20):
    """Served shot stream: Poisson arrivals of ``njobs`` jobs, 70 % modeling
    and 30 % RTM, grids drawn uniformly from SERVED_GRIDS at 10 m, record
    lengths from SERVED_SECONDS at dt = 1 ms, Ricker 10-30 Hz, random
    layered-plus-Gaussian-anomaly models in 1500-4500 m/s (a seeded pool of
    ``models_per_grid`` per grid; migration models are their 9-point Gaussian
    smoothing).  The arrival rate (jobs/s) is drawn from the seed in [10, 20]
    unless given.  Returns (schedule, pools) where pools[grid] = [(v, vs)]."""
    rng = np.random.default_rng(seed)
    rate = float(rng.uniform(10.0, 20.0)) if rate is None else float(rate)
    h = 10.0
    pools = {}
    for g in SERVED_GRIDS:
        pools[g] = []
        for _ in range(models_per_grid):
            v = layered_anomaly_model(g[0], g[1], h, rng)
            pools[g].append((v, gaussian_smooth(v, 9)))
    t = 0.0
    sched = []
    for _ in range(njobs):
        t += float(rng.exponential(1.0 / rate))
        g = SERVED_GRIDS[int(rng.integers(len(SERVED_GRIDS)))]
        kind = "model" if rng.random() < 0.7 else "rtm"
        nt = int(round(SERVED_SECONDS[int(rng.integers(len(SERVED_SECONDS)))] / 1e-3))
        sched.append(ServedJob(t, kind, g, nt, float(rng.uniform(10.0, 30.0)), int(rng.integers(models_per_grid)),
                               int(rng.integers(d_pml + 2, g[1] - d_pml))))
    return sched, pools, rate


def served_shot_job(sj: ServedJob, pools, d_pml: int = 20):
    """ShotJob of one stream entry: source one row below the CPML at column
    ``xs``, receivers on every column of the first physical row + 1."""
    from .api import ShotJob
    v, vs = pools[sj.grid][sj.model]
    nz, nx = sj.grid
    xr = np.arange(d_pml + 1, nx - d_pml + 1, dtype=np.float64)
    zr = np.full(xr.size, float(d_pml + 2))
    return ShotJob(kind=sj.kind, v=v, vs=vs if sj.kind == "rtm" else None, dx=10.0, dz=10.0, dt=1e-3, nt=sj.nt,
                   d_pml=d_pml, zs=float(d_pml + 2), xs=float(sj.xs), zr=zr, xr=xr, w=ricker(sj.fc, 1e-3, sj.nt),
                   keep_data=True)


# ---------------------------------------------------------------------------
# Acquisition geometry and model smoothing of the reference's drivers

def acquisi(V, dx, dz, zsc, zrc, h_offset, ds, dr, slag, rlag, acq_type: str = "fixspread", manual=None):
    """Source and receiver positions in metres, as ``SRC/MNAD/acquisi.m``.

    ``V`` is the unpadded model (nz x nx); ``zsc`` / ``zrc`` source and
    receiver depths, ``h_offset`` the half offset, ``ds`` / ``dr`` the source
    and receiver spacings, ``slag`` / ``rlag`` the edge margins (metres).
    ``acq_type``: 'fixspread', 'onesided', 'splitspread', 'obn' (sources on
    the sea floor below a constant-velocity water column, receivers at
    ``zsc``) or 'arbitrary' (``manual`` = dict of grid indices xs, zs, xr,
    zr).  Returns ``(Source, Receiver)``: Source is 2 x ns (x; z), Receiver
    a list of ns (x_metres, z_metres) pairs.  Grid indices are 1-based and
    unpadded; the drivers add d_pml (``padded_indices``)."""
    V = np.asarray(V, dtype=np.float64)
    nz, nx = V.shape
    ds = int(np.trunc(ds / dx)) or 1
    dr = int(np.trunc(dr / dx)) or 1
    kind = acq_type.lower()

    def rng(a, step, b):
        return np.arange(a, b + 1, step, dtype=np.float64) if b >= a else np.zeros(0)

    if kind == "arbitrary":
        if manual is None:
            raise ValueError("acqType is 'arbitrary' but manualGeom was not provided")
        for key in ("xs", "zs", "xr", "zr"):
            if key not in manual:
                raise ValueError(f"manualGeom is missing required field '{key}'")
        xs = np.asarray(manual["xs"], dtype=np.float64).ravel()
        zs = np.asarray(manual["zs"], dtype=np.float64).ravel()
        xr = [np.asarray(x, dtype=np.float64).ravel() for x in manual["xr"]]
        zr = [np.asarray(z, dtype=np.float64).ravel() for z in manual["zr"]]
    else:
        xs = rng(math.ceil(slag / dx), ds, nx - math.floor(slag / dx))
        zs = np.zeros_like(xs) + math.floor(zsc / dz)
        h_off = math.floor(h_offset / dx)
        last = nx - math.floor(rlag / dx)
        xr, zr = [], []
        if kind == "obn":
            water = V[0, 0]
            xs = rng(math.ceil(rlag / dx), dr, last)
            zs = np.array([float(np.flatnonzero(V[:, int(x) - 1] == water).max() + 1) for x in xs])
            for _ in xs:
                r = rng(math.ceil(slag / dx), ds, nx - math.floor(slag / dx))
                xr.append(r)
                zr.append(0.0 * r + math.floor(zsc / dz))
        else:
            for s in xs:
                if kind == "onesided":
                    r = rng(s, dr, last) if s + h_off > last else rng(s, dr, s + h_off - 1)
                elif kind == "splitspread":
                    if s + h_off > last:
                        r = rng(s - h_off, dr, last)
                    elif s - h_off <= 0:
                        r = rng(1, dr, s + h_off - 1)
                    else:
                        r = rng(s - h_off, dr, s + h_off - 1)
                elif kind == "fixspread":
                    r = rng(math.ceil(rlag / dx), dr, last)
                else:
                    raise ValueError(f"unknown acqType {acq_type!r}; use 'splitspread', 'onesided', 'obn', "
                                     "'fixspread' or 'arbitrary'")
                xr.append(r)
                zr.append(0.0 * r + math.floor(zrc / dz))
    Source = np.vstack([dx * xs, dz * zs])
    Receiver = [(dx * x, dz * z) for x, z in zip(xr, zr)]
    return Source, Receiver


def padded_indices(Source, Receiver, dx, dz, d_pml):
    """1-based padded grid indices of the drivers (``main_Acoustic_RTM.m:124-130``):
    index = d_pml + metres / spacing.  Returns (xs, zs, [xr], [zr])."""
    xs = d_pml + np.asarray(Source[0]) / dx
    zs = d_pml + np.asarray(Source[1]) / dz
    return xs, zs, [d_pml + x / dx for x, _ in Receiver], [d_pml + z / dz for _, z in Receiver]


def v_smooth(v, s1: int, s2: int, nit: int) -> np.ndarray:
    """Smoothed migration model of ``SRC/MNAD/v_smooth.m``: ``nit`` passes of
    an s1 x s2 box average of the slowness with edge replication."""
    s0 = 1.0 / np.asarray(v, dtype=np.float64)
    h1, h2 = (s1 - 1) // 2, (s2 - 1) // 2
    n1, n2 = s0.shape
    for _ in range(nit):
        p = np.pad(s0, ((h1, h1), (h2, h2)), mode="edge")
        # window sums: columns first, then rows, as sum(sum(window))
        cz = np.zeros((p.shape[0] - 2 * h1, p.shape[1]))
        for a in range(s1):
            cz += p[a:a + n1, :]
        acc = np.zeros((n1, n2))
        for b in range(s2):
            acc += cz[:, b:b + n2]
        s0 = acc / (s1 * s2)
    return 1.0 / s0
