"""FP64 CPU oracle for the MNAD modeling / RTM hot path -- TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may
import it.  The product path (the CUDA library behind ``include/mnad.h``)
never calls into ``oracle/``.

What it is: a literal NumPy/SciPy restatement of the reference MATLAB code
(Ahmadreza205/MNAD-Modeling-RTM).  The nine MNAD operators are assembled as
sparse N x N matrices from the same ``I``/``J`` index arrays and the same
coefficient expressions as ``SRC/MNAD/A??_gen.m``; the CPML coefficients and
memory recurrences follow ``SRC/MNAD/C_cof.m``, ``SRC/MNAD/Ux123_gen.m`` and
``SRC/MNAD/Uz123_gen.m``; the time loops follow
``SRC/MNAD/fwd_PDE_exact_MNAD.m`` and ``SRC/migration/Born_adj_MNAD.m`` step
for step, with these documented decisions:

* ``Born_adj_MNAD.m:105-106`` names an undefined variable ``U_r``; it is read
  as ``U`` (the forward update at ``fwd_PDE_exact_MNAD.m:115-116``).
* ``Born_adj_MNAD.m:50`` expects a cell; ``data`` may be a list (``[0]`` is
  used) or an ``nt x nr`` array.
* The display call at ``fwd_PDE_exact_MNAD.m:155`` is dropped (headless).
* Snapshot pairing follows the reference exactly: the snapshot matrix has
  ``ncols = max(2*nf+1, k)`` columns, of which the first ``k`` are filled; the
  adjoint pairs column ``ncols-ttt+1`` (``Born_adj_MNAD.m:128``).  Columns past
  ``k`` are zero.  ``pairing="aligned"`` pairs column ``k-ttt+1`` instead.

Pinning: the reference is MATLAB and ships no golden vectors or tests, and
neither MATLAB nor GNU Octave is available.  Its own ``.m`` sources were run
under the MATLAB-subset interpreter ``oracle/mlite.py``
(``tests/golden/make_reference_golden.py``); this restatement reproduces those
runs (``tests/golden/golden_ref_*.npz``) to 1e-12 (``tests/test_reference_golden.py``).
It is also cross-checked against the independent matrix-free FP64 C
restatement (``oracle/mnad_oracle.c``) to ~1e-13.

Indexing: arrays have MATLAB shape ``(nz, nx)`` (z = row, x = column) and
are flattened column-major (``order="F"``), matching ``idx(j,i)=j+(i-1)*nz``
(``SRC/MNAD/Auu_gen.m:22``).  Source/receiver indices are 1-based like the
MATLAB call signature.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

__all__ = [
    "a_gen", "c_cof", "ux123_gen", "uz123_gen", "snapshot_plan", "snapshot_nf",
    "fwd_pde_exact_mnad", "born_adj_mnad", "ricker", "pad_model", "v_smooth",
    "acquisi",
]

_NAMES = ("Auu", "Auv", "Auw", "Avu", "Avv", "Avw", "Awu", "Awv", "Aww")


# ---------------------------------------------------------------------------
# Operators (SRC/MNAD/A??_gen.m)
# ---------------------------------------------------------------------------
def _entries(v, nz, nx, jr, ir, dj, di):
    """Row/col indices of one stencil entry.

    ``jr``/``ir`` are the 0-based destination row/column ranges (the MATLAB
    ``j = ...; i = ...`` lines); the source point is ``(j+dj, i+di)``.
    Returns (I, J, vsub) flattened column-major like ``I1(:)``.
    """
    idx = np.arange(nz * nx).reshape((nz, nx), order="F")
    jj = np.arange(*jr)
    ii = np.arange(*ir)
    I = idx[np.ix_(jj, ii)].ravel(order="F")
    J = idx[np.ix_(jj + dj, ii + di)].ravel(order="F")
    vs = v[np.ix_(jj, ii)]
    return I, J, vs


def _assemble(nz, nx, parts):
    I = np.concatenate([p[0] for p in parts])
    J = np.concatenate([p[1] for p in parts])
    V = np.concatenate([p[2].ravel(order="F") for p in parts])
    n = nz * nx
    return sp.csr_matrix((V, (I, J)), shape=(n, n))


def a_gen(dx, dz, dt, v):
    """Assemble the nine MNAD operators; returns a dict keyed Auu..Aww.

    Each block restates one ``A??_gen.m`` file: the ``(dj, di)`` offsets are
    taken from its ``J = idx(j+dj, i+di)`` lines (not from its comments, some
    of which are mirrored) and the coefficient is the file's expression in
    the destination velocity ``v(j,i)``.
    """
    v = np.asarray(v, dtype=np.float64)
    nz, nx = v.shape
    Z, X = nz, nx
    fz, fx = (0, Z), (0, X)            # j = 1:nz  /  i = 1:nx
    zlo, zhi = (1, Z), (0, Z - 1)      # j = 2:nz  /  j = 1:nz-1
    xlo, xhi = (1, X), (0, X - 1)      # i = 2:nx  /  i = 1:nx-1
    ops = {}

    def E(jr, ir, dj, di, f):
        I, J, vs = _entries(v, nz, nx, jr, ir, dj, di)
        return I, J, f(vs)

    # Auu_gen.m:26-86
    ops["Auu"] = _assemble(nz, nx, [
        E(zlo, fx, -1, 0, lambda a: (24/11)*a**2*dt**2/dz**2 - a**4*dt**4*(15/(11*dz**4) + 1/(dx**2*dz**2))),
        E(fz, xlo, 0, -1, lambda a: (24/11)*a**2*dt**2/dx**2 - a**4*dt**4*(15/(11*dx**4) + 1/(dx**2*dz**2))),
        E(fz, fx, 0, 0, lambda a: 2 - (48/11)*a**2*dt**2*(1/dx**2 + 1/dz**2) + (30/11)*a**4*dt**4*(1/dx**4 + 1/dz**4 + 11/(15*dx**2*dz**2))),
        E(fz, xhi, 0, 1, lambda a: (24/11)*a**2*dt**2/dx**2 - a**4*dt**4*(15/(11*dx**4) + 1/(dx**2*dz**2))),
        E(zhi, fx, 1, 0, lambda a: (24/11)*a**2*dt**2/dz**2 - a**4*dt**4*(15/(11*dz**4) + 1/(dx**2*dz**2))),
        E(zlo, xlo, -1, -1, lambda a: a**4*dt**4/(2*dx**2*dz**2)),
        E(zhi, xlo, 1, -1, lambda a: a**4*dt**4/(2*dx**2*dz**2)),
        E(zlo, xhi, -1, 1, lambda a: a**4*dt**4/(2*dx**2*dz**2)),
        E(zhi, xhi, 1, 1, lambda a: a**4*dt**4/(2*dx**2*dz**2)),
    ])
    # Auv_gen.m:25-78
    ops["Auv"] = _assemble(nz, nx, [
        E(fz, xlo, 0, -1, lambda a: (-20/33)*a**2*dt**2/dx + a**4*dt**4*(47/(66*dx**3) + 1/(6*dx*dz**2))),
        E(fz, xhi, 0, 1, lambda a: (20/33)*a**2*dt**2/dx - a**4*dt**4*(47/(66*dx**3) + 1/(6*dx*dz**2))),
        E(zlo, xlo, -1, -1, lambda a: -a**4*dt**4/(12*dx*dz**2)),
        E(zhi, xlo, 1, -1, lambda a: -a**4*dt**4/(12*dx*dz**2)),
        E(zlo, xhi, -1, 1, lambda a: a**4*dt**4/(12*dx*dz**2)),
        E(zhi, xhi, 1, 1, lambda a: a**4*dt**4/(12*dx*dz**2)),
        E(fz, (2, X), 0, -2, lambda a: (1/132)*a**2*dt**2/dx - (1/66)*a**4*dt**4/dx**3),
        E(fz, (0, X - 2), 0, 2, lambda a: (-1/132)*a**2*dt**2/dx + (1/66)*a**4*dt**4/dx**3),
    ])
    # Auw_gen.m:25-78
    ops["Auw"] = _assemble(nz, nx, [
        E(zhi, fx, 1, 0, lambda a: (20/33)*a**2*dt**2/dz - a**4*dt**4*(47/(66*dz**3) + 1/(6*dz*dx**2))),
        E(zlo, fx, -1, 0, lambda a: (-20/33)*a**2*dt**2/dz + a**4*dt**4*(47/(66*dz**3) + 1/(6*dz*dx**2))),
        E(zlo, xlo, -1, -1, lambda a: -a**4*dt**4/(12*dz*dx**2)),
        E(zhi, xlo, 1, -1, lambda a: a**4*dt**4/(12*dz*dx**2)),
        E(zlo, xhi, -1, 1, lambda a: -a**4*dt**4/(12*dz*dx**2)),
        E(zhi, xhi, 1, 1, lambda a: a**4*dt**4/(12*dz*dx**2)),
        E((0, Z - 2), fx, 2, 0, lambda a: (-1/132)*a**2*dt**2/dz + (1/66)*a**4*dt**4/dz**3),
        E((2, Z), fx, -2, 0, lambda a: (1/132)*a**2*dt**2/dz - (1/66)*a**4*dt**4/dz**3),
    ])
    # Avu_gen.m:26-65
    ops["Avu"] = _assemble(nz, nx, [
        E(fz, xlo, 0, -1, lambda a: -a**4*dt**4*(15/(2*dx**5) - 1/(dx*dz**4) + 5/(2*dx**3*dz**2)) + a**2*dt**2*(15/(2*dx**3) - 1/(dx*dz**2))),
        E(fz, xhi, 0, 1, lambda a: a**4*dt**4*(15/(2*dx**5) - 1/(dx*dz**4) + 5/(2*dx**3*dz**2)) - a**2*dt**2*(15/(2*dx**3) - 1/(dx*dz**2))),
        E(zlo, xlo, -1, -1, lambda a: a**4*dt**4*(5/(4*dx**3*dz**2) - 1/(2*dx*dz**4)) + a**2*dt**2/(2*dx*dz**2)),
        E(zhi, xlo, 1, -1, lambda a: a**4*dt**4*(5/(4*dx**3*dz**2) - 1/(2*dx*dz**4)) + a**2*dt**2/(2*dx*dz**2)),
        E(zlo, xhi, -1, 1, lambda a: -a**4*dt**4*(5/(4*dx**3*dz**2) - 1/(2*dx*dz**4)) - a**2*dt**2/(2*dx*dz**2)),
        E(zhi, xhi, 1, 1, lambda a: -a**4*dt**4*(5/(4*dx**3*dz**2) - 1/(2*dx*dz**4)) - a**2*dt**2/(2*dx*dz**2)),
    ])
    # Avv_gen.m:25-85
    ops["Avv"] = _assemble(nz, nx, [
        E(zlo, fx, -1, 0, lambda a: a**2*dt**2/dz**2 - 2*a**4*dt**4/(dx**2*dz**2)),
        E(fz, xlo, 0, -1, lambda a: -(3/2)*a**2*dt**2/dx**2 + a**4*dt**4*(5/(2*dx**4) + 1/(2*dx**2*dz**2))),
        E(fz, fx, 0, 0, lambda a: 2 - a**2*dt**2*(12/dx**2 + 2/dz**2) + a**4*dt**4*(10/dx**4 + 4/(dx**2*dz**2))),
        E(fz, xhi, 0, 1, lambda a: -(3/2)*a**2*dt**2/dx**2 + a**4*dt**4*(5/(2*dx**4) + 1/(2*dx**2*dz**2))),
        E(zhi, fx, 1, 0, lambda a: a**2*dt**2/dz**2 - 2*a**4*dt**4/(dx**2*dz**2)),
        E(zlo, xlo, -1, -1, lambda a: -a**4*dt**4/(4*dx**2*dz**2)),
        E(zhi, xlo, 1, -1, lambda a: -a**4*dt**4/(4*dx**2*dz**2)),
        E(zlo, xhi, -1, 1, lambda a: -a**4*dt**4/(4*dx**2*dz**2)),
        E(zhi, xhi, 1, 1, lambda a: -a**4*dt**4/(4*dx**2*dz**2)),
    ])
    # Avw_gen.m:25-50
    ops["Avw"] = _assemble(nz, nx, [
        E(zlo, xlo, -1, -1, lambda a: a**4*dt**4/(4*dz**3*dx) - a**2*dt**2/(4*dz*dx)),
        E(zhi, xlo, 1, -1, lambda a: -a**4*dt**4/(4*dz**3*dx) + a**2*dt**2/(4*dz*dx)),
        E(zlo, xhi, -1, 1, lambda a: -a**4*dt**4/(4*dz**3*dx) + a**2*dt**2/(4*dz*dx)),
        E(zhi, xhi, 1, 1, lambda a: a**4*dt**4/(4*dz**3*dx) - a**2*dt**2/(4*dz*dx)),
    ])
    # Awu_gen.m:25-67
    ops["Awu"] = _assemble(nz, nx, [
        E(zlo, fx, -1, 0, lambda a: -a**4*dt**4*(15/(2*dz**5) - 1/(dz*dx**4) + 5/(2*dz**3*dx**2)) + a**2*dt**2*(15/(2*dz**3) - 1/(dz*dx**2))),
        E(zhi, fx, 1, 0, lambda a: a**4*dt**4*(15/(2*dz**5) - 1/(dz*dx**4) + 5/(2*dz**3*dx**2)) - a**2*dt**2*(15/(2*dz**3) - 1/(dz*dx**2))),
        E(zlo, xlo, -1, -1, lambda a: a**4*dt**4*(5/(4*dz**3*dx**2) - 1/(2*dz*dx**4)) + a**2*dt**2*(1/(2*dz*dx**2))),
        E(zhi, xlo, 1, -1, lambda a: -a**4*dt**4*(5/(4*dz**3*dx**2) - 1/(2*dz*dx**4)) - a**2*dt**2*(1/(2*dz*dx**2))),
        E(zlo, xhi, -1, 1, lambda a: a**4*dt**4*(5/(4*dz**3*dx**2) - 1/(2*dz*dx**4)) + a**2*dt**2*(1/(2*dz*dx**2))),
        E(zhi, xhi, 1, 1, lambda a: -a**4*dt**4*(5/(4*dz**3*dx**2) - 1/(2*dz*dx**4)) - a**2*dt**2*(1/(2*dz*dx**2))),
    ])
    # Awv_gen.m:27-52
    ops["Awv"] = _assemble(nz, nx, [
        E(zlo, xlo, -1, -1, lambda a: a**4*dt**4/(4*dx**3*dz) - a**2*dt**2/(4*dz*dx)),
        E(zhi, xlo, 1, -1, lambda a: -a**4*dt**4/(4*dx**3*dz) + a**2*dt**2/(4*dz*dx)),
        E(zlo, xhi, -1, 1, lambda a: -a**4*dt**4/(4*dx**3*dz) + a**2*dt**2/(4*dz*dx)),
        E(zhi, xhi, 1, 1, lambda a: a**4*dt**4/(4*dx**3*dz) - a**2*dt**2/(4*dz*dx)),
    ])
    # Aww_gen.m:27-87
    ops["Aww"] = _assemble(nz, nx, [
        E(zlo, fx, -1, 0, lambda a: -(3/2)*a**2*dt**2/dz**2 + a**4*dt**4*(5/(2*dz**4) + 1/(2*dx**2*dz**2))),
        E(fz, xlo, 0, -1, lambda a: a**2*dt**2/dx**2 - 2*a**4*dt**4/(dz**2*dx**2)),
        E(fz, fx, 0, 0, lambda a: 2 - a**2*dt**2*(12/dz**2 + 2/dx**2) + a**4*dt**4*(10/dz**4 + 4/(dx**2*dz**2))),
        E(fz, xhi, 0, 1, lambda a: a**2*dt**2/dx**2 - 2*a**4*dt**4/(dz**2*dx**2)),
        E(zhi, fx, 1, 0, lambda a: -(3/2)*a**2*dt**2/dz**2 + a**4*dt**4*(5/(2*dz**4) + 1/(2*dx**2*dz**2))),
        E(zlo, xlo, -1, -1, lambda a: -a**4*dt**4/(4*dx**2*dz**2)),
        E(zhi, xlo, 1, -1, lambda a: -a**4*dt**4/(4*dx**2*dz**2)),
        E(zlo, xhi, -1, 1, lambda a: -a**4*dt**4/(4*dx**2*dz**2)),
        E(zhi, xhi, 1, 1, lambda a: -a**4*dt**4/(4*dx**2*dz**2)),
    ])
    return ops


# ---------------------------------------------------------------------------
# CPML (SRC/MNAD/C_cof.m, Ux123_gen.m, Uz123_gen.m)
# ---------------------------------------------------------------------------
def c_cof(R, d_pml, dx, dz, dt, nx, nz, v):
    """The 12 CPML coefficient fields of ``SRC/MNAD/C_cof.m:1-67`` (dense)."""
    v = np.asarray(v, dtype=np.float64)
    d = d_pml
    out = {}
    # X accessories (C_cof.m:4-33)
    D = d * dx
    x_b = np.concatenate([D - dx * np.arange(d), np.zeros(nx - 2 * d), dx * np.arange(1, d + 1)])
    X = np.tile(x_b, (nz, 1))
    K = (3 * math.log(1 / R)) / (2 * D**3)
    for side, cols in (("xl", slice(d, nx)), ("xr", slice(0, nx - d))):
        Vs = v.copy()
        Vs[:, cols] = 0
        sig0 = K * Vs
        sig = sig0 * (X**2)
        dsig = 2 * sig0 * X
        den = 1 + sig * (dt / 2)
        out["c1" + side] = (1 - sig * (dt / 2)) / den
        out["c2" + side] = (dsig * dt) / den
        out["c3" + side] = (sig * dt) / den
    # Z accessories (C_cof.m:35-65)
    D = d * dz
    z_b = np.concatenate([D - dz * np.arange(d), np.zeros(nz - 2 * d), dz * np.arange(1, d + 1)])
    Zm = np.tile(z_b[:, None], (1, nx))
    K = (3 * math.log(1 / R)) / (2 * D**3)
    for side, rows in (("zt", slice(d, nz)), ("zb", slice(0, nz - d))):
        Vs = v.copy()
        Vs[rows, :] = 0
        sig0 = K * Vs
        sig = sig0 * (Zm**2)
        dsig = 2 * sig0 * Zm
        den = 1 + sig * (dt / 2)
        out["c1" + side] = (1 - sig * (dt / 2)) / den
        out["c2" + side] = (dsig * dt) / den
        out["c3" + side] = (sig * dt) / den
    return out


def ux123_gen(M, U, dx, c):
    """``SRC/MNAD/Ux123_gen.m``: update the x memory variables of one field.

    ``M`` is a dict with keys ``1xl 2xl 3xl 1xr 2xr 3xr`` updated in place;
    returns ``F1_x = M1xl + M1xr``.
    """
    nz, nx = U.shape
    Ua = np.zeros_like(U)
    Ua[:, : nx - 1] = U[:, 1:]
    Ud = np.zeros_like(U)
    Ud[:, 1:] = U[:, : nx - 1]
    c1, c2, c3 = c["c1xl"], c["c2xl"], c["c3xl"]
    M["3xl"] = c1 * M["3xl"] + (c2 / (2 * dx)) * (Ud - Ua)
    M["2xl"] = c1 * M["2xl"] + (c2 / dx) * (Ud - Ua) + c3 * ((Ud - 2 * U + Ua) / (dx**2) - M["3xl"])
    M["1xl"] = c1 * M["1xl"] + (c2 / (2 * dx)) * (Ud - Ua) + c3 * (2 * (Ud - 2 * U + Ua) / (dx**2) - M["2xl"])
    c1, c2, c3 = c["c1xr"], c["c2xr"], c["c3xr"]
    M["3xr"] = c1 * M["3xr"] + (c2 / (2 * dx)) * (Ua - Ud)
    M["2xr"] = c1 * M["2xr"] + (c2 / dx) * (Ua - Ud) + c3 * ((Ua - 2 * U + Ud) / (dx**2) - M["3xr"])
    M["1xr"] = c1 * M["1xr"] + (c2 / (2 * dx)) * (Ua - Ud) + c3 * (2 * (Ua - 2 * U + Ud) / (dx**2) - M["2xr"])
    return M["1xl"] + M["1xr"]


def uz123_gen(M, U, dz, c):
    """``SRC/MNAD/Uz123_gen.m``: update the z memory variables of one field."""
    nz, nx = U.shape
    Ua = np.zeros_like(U)
    Ua[: nz - 1, :] = U[1:, :]
    Ud = np.zeros_like(U)
    Ud[1:, :] = U[: nz - 1, :]
    c1, c2, c3 = c["c1zt"], c["c2zt"], c["c3zt"]
    M["3zt"] = c1 * M["3zt"] + (c2 / (2 * dz)) * (Ud - Ua)
    M["2zt"] = c1 * M["2zt"] + (c2 / dz) * (Ud - Ua) + c3 * ((Ud - 2 * U + Ua) / (dz**2) - M["3zt"])
    M["1zt"] = c1 * M["1zt"] + (c2 / (2 * dz)) * (Ud - Ua) + c3 * (2 * (Ud - 2 * U + Ua) / (dz**2) - M["2zt"])
    c1, c2, c3 = c["c1zb"], c["c2zb"], c["c3zb"]
    M["3zb"] = c1 * M["3zb"] + (c2 / (2 * dz)) * (Ua - Ud)
    M["2zb"] = c1 * M["2zb"] + (c2 / dz) * (Ua - Ud) + c3 * ((Ua - 2 * U + Ud) / (dz**2) - M["3zb"])
    M["1zb"] = c1 * M["1zb"] + (c2 / (2 * dz)) * (Ua - Ud) + c3 * (2 * (Ua - 2 * U + Ud) / (dz**2) - M["2zb"])
    return M["1zb"] + M["1zt"]


def _new_mem(nz, nx):
    keys = ("1xl", "2xl", "3xl", "1xr", "2xr", "3xr", "1zt", "2zt", "3zt", "1zb", "2zb", "3zb")
    return {k: np.zeros((nz, nx)) for k in keys}


def snapshot_nf(v, nt):
    """``nf`` of ``fwd_PDE_exact_MNAD.m:46`` (same operation order)."""
    v = np.asarray(v, dtype=np.float64)
    return math.floor(nt / (2 * 3 * float(v.max()) / float(v.min())))


def snapshot_plan(v, nt):
    """``(nf, T)`` exactly as ``fwd_PDE_exact_MNAD.m:46-47`` computes them.

    Raises ZeroDivisionError when ``nf == 0`` (the reference divides by zero
    there).
    """
    nf = snapshot_nf(v, nt)
    if nf == 0:
        raise ZeroDivisionError("nf == 0: T = floor(nt/nf/2) is undefined")
    T = math.floor(nt / nf / 2)
    return nf, T


def _apply(A, F):
    nz, nx = F.shape
    return (A @ F.ravel(order="F")).reshape((nz, nx), order="F")


# ---------------------------------------------------------------------------
# Forward propagator (SRC/MNAD/fwd_PDE_exact_MNAD.m)
# ---------------------------------------------------------------------------
def fwd_pde_exact_mnad(dx, xs, xr, dz, zs, zr, v, dt, nt, w, d_pml, ss=1, A=None,
                       indx=0, T=None, record_vw=False, keep_steps=()):
    """One shot forward in time; mirrors ``fwd_PDE_exact_MNAD.m:1-168``.

    Returns a dict with ``datau`` (nt x nr), ``datav``/``dataw`` when
    ``record_vw``, and with ``indx == 1`` the snapshot matrix ``UU``
    (Nint x ncols, ncols = max(2nf+1, k)), ``illum`` ((nz-2d) x (nx-2d),
    already multiplied by T as in ``:162``), ``T``, ``nf``, ``k``.
    ``keep_steps`` lists time steps tt (1-based) whose new field ``nU`` is
    returned in ``fields[tt]`` as (nU, nV, nW).
    """
    v = np.asarray(v, dtype=np.float64)
    nz, nx = v.shape
    if A is None:
        A = a_gen(dx, dz, dt, v)
    xr = np.asarray(xr).astype(int).ravel()
    zr = np.asarray(zr).astype(int).ravel()
    xs, zs = int(xs), int(zs)
    w = np.asarray(w, dtype=np.float64).ravel()
    V2dt2 = v**2 * (dt**2)                                   # :39
    d = d_pml
    out = {}
    if indx == 1:
        if T is None:
            nf, T = snapshot_plan(v, nt)                       # :46-47
        else:
            nf = snapshot_nf(v, nt)
        nint = (nz - 2 * d) * (nx - 2 * d)
        k = nt // T
        ncols = max(2 * nf + 1, k)
        UU = np.zeros((nint, ncols))                           # :53
        ttt = 0
        illum = np.zeros((nz - 2 * d, nx - 2 * d))
    nr = len(xr)
    datau = np.zeros((nt, nr))
    datav = np.zeros((nt, nr)) if record_vw else None
    dataw = np.zeros((nt, nr)) if record_vw else None
    pU = np.zeros((nz, nx)); U = np.zeros((nz, nx))
    pV = np.zeros((nz, nx)); V = np.zeros((nz, nx))
    pW = np.zeros((nz, nx)); W = np.zeros((nz, nx))
    MU, MV, MW = _new_mem(nz, nx), _new_mem(nz, nx), _new_mem(nz, nx)
    c = c_cof(1e-4, d, dx, dz, dt, nx, nz, v)                  # :88-89
    fields = {}
    for tt in range(1, nt + 1):                                # :92
        U1x = ux123_gen(MU, U, dx, c); U1z = uz123_gen(MU, U, dz, c)
        V1x = ux123_gen(MV, V, dx, c); V1z = uz123_gen(MV, V, dz, c)
        W1x = ux123_gen(MW, W, dx, c); W1z = uz123_gen(MW, W, dz, c)
        U[zs - 1, xs - 1] = U[zs - 1, xs - 1] + V2dt2[zs - 1, xs - 1] * w[tt - 1]   # :111
        nU = _apply(A["Auu"], U) + _apply(A["Auv"], V) + _apply(A["Auw"], W) - pU - V2dt2 * (U1x + U1z)
        nV = _apply(A["Avv"], V) + _apply(A["Avu"], U) + _apply(A["Avw"], W) - pV - V2dt2 * (V1x + V1z)
        nW = _apply(A["Aww"], W) + _apply(A["Awu"], U) + _apply(A["Awv"], V) - pW - V2dt2 * (W1x + W1z)
        datau[tt - 1, :] = U[zr - 1, xr - 1]                    # :119-123
        if record_vw:
            datav[tt - 1, :] = V[zr - 1, xr - 1]
            dataw[tt - 1, :] = W[zr - 1, xr - 1]
        if indx == 1:                                          # :126-143
            if tt == 1:
                d2u = nU / dt**2
            elif tt == 2:
                d2u = (nU - 2 * U) / dt**2
            else:
                d2u = (nU - 2 * U + pU) / dt**2
            if tt % T == 0:
                internal = d2u[d:nz - d, d:nx - d]
                UU[:, ttt] = internal.ravel(order="F")
                illum = illum + internal**2
                ttt += 1
        if tt in keep_steps:
            fields[tt] = (nU.copy(), nV.copy(), nW.copy())
        pU, U = U, nU                                          # :146-153
        pV, V = V, nV
        pW, W = W, nW
    out["datau"] = datau
    if record_vw:
        out["datav"], out["dataw"] = datav, dataw
    if indx == 1:
        out.update(UU=UU, illum=T * illum, T=T, nf=nf, k=k)    # :160-164
    out["fields"] = fields
    out["final"] = (pU, U, pV, V, pW, W)
    return out


# ---------------------------------------------------------------------------
# Adjoint / RTM propagator (SRC/migration/Born_adj_MNAD.m)
# ---------------------------------------------------------------------------
def born_adj_mnad(dx, dz, nt, dt, v, xr, zr, data, d_pml, UU, A=None, T=None,
                  pairing="reference", nf=None):
    """Reverse-time propagation + zero-lag imaging; ``Born_adj_MNAD.m:1-140``.

    ``UU`` is the forward snapshot matrix (what ``load UU_<ss>`` provides at
    ``:33``).  Returns ``Im`` (Nint,) = T * sum(US .* UR) (``:138``).
    """
    v = np.asarray(v, dtype=np.float64)
    nz, nx = v.shape
    if A is None:
        A = a_gen(dx, dz, dt, v)
    if isinstance(data, (list, tuple)):                        # :50 (cell)
        data = data[0]
    datau = np.asarray(data, dtype=np.float64)
    xr = np.asarray(xr).astype(int).ravel()
    zr = np.asarray(zr).astype(int).ravel()
    V2dt2 = (v * dt)**2                                        # :36
    if T is None:
        nf, T = snapshot_plan(v, nt)                           # :41-42
    d = d_pml
    ncols = UU.shape[1]
    k = nt // T
    Im = np.zeros((nz - 2 * d) * (nx - 2 * d))
    ttt = 0
    pU = np.zeros((nz, nx)); U = np.zeros((nz, nx))
    pV = np.zeros((nz, nx)); V = np.zeros((nz, nx))
    pW = np.zeros((nz, nx)); W = np.zeros((nz, nx))
    MU, MV, MW = _new_mem(nz, nx), _new_mem(nz, nx), _new_mem(nz, nx)
    c = c_cof(1e-4, d, dx, dz, dt, nx, nz, v)                  # :81-82
    for tt in range(nt, 0, -1):                                # :85
        U1x = ux123_gen(MU, U, dx, c); U1z = uz123_gen(MU, U, dz, c)
        V1x = ux123_gen(MV, V, dx, c); V1z = uz123_gen(MV, V, dz, c)
        W1x = ux123_gen(MW, W, dx, c); W1z = uz123_gen(MW, W, dz, c)
        nU = _apply(A["Auu"], U) + _apply(A["Auv"], V) + _apply(A["Auw"], W) - pU - V2dt2 * (U1x + U1z)
        nV = _apply(A["Avv"], V) + _apply(A["Avu"], U) + _apply(A["Avw"], W) - pV - V2dt2 * (V1x + V1z)
        nW = _apply(A["Aww"], W) + _apply(A["Awu"], U) + _apply(A["Awv"], V) - pW - V2dt2 * (W1x + W1z)
        for rr in range(len(xr)):                              # :109-111
            U[zr[rr] - 1, xr[rr] - 1] = U[zr[rr] - 1, xr[rr] - 1] + V2dt2[zr[rr] - 1, xr[rr] - 1] * datau[tt - 1, rr]
        pU, U = U, nU                                          # :116-123
        pV, V = V, nV
        pW, W = W, nW
        if tt % T == 0:                                        # :127-134
            col = (ncols - ttt) if pairing == "reference" else (k - ttt)
            US = UU[:, col - 1] if 1 <= col <= ncols else 0.0
            UR = U[d:nz - d, d:nx - d].ravel(order="F")
            Im = Im + US * UR
            ttt += 1
    return T * Im                                              # :138


# ---------------------------------------------------------------------------
# Workflow helpers (driver-side, SRC/migration/main_Acoustic_RTM.m)
# ---------------------------------------------------------------------------
def ricker(fc, dt, nt):
    """Ricker wavelet of ``main_Acoustic_RTM.m:138-140`` sampled at t=(0:nt-1)dt."""
    t = np.arange(nt) * dt
    t0 = 1.1 / fc
    tau = np.pi * (t - t0) * fc
    return (1 - 2 * tau**2) * np.exp(-tau**2)


def pad_model(V, d_pml):
    """Edge-replicated padding of ``main_Acoustic_RTM.m:148-149``."""
    V = np.asarray(V, dtype=np.float64)
    v = np.concatenate([np.repeat(V[:, :1], d_pml, 1), V, np.repeat(V[:, -1:], d_pml, 1)], 1)
    return np.concatenate([np.repeat(v[:1, :], d_pml, 0), v, np.repeat(v[-1:, :], d_pml, 0)], 0)


def v_smooth(v, s1, s2, nit):
    """Box filter on slowness with edge replication (``SRC/MNAD/v_smooth.m``)."""
    s0 = 1.0 / np.asarray(v, dtype=np.float64)
    h1, h2 = (s1 - 1) // 2, (s2 - 1) // 2
    n1, n2 = s0.shape
    for _ in range(nit):
        p = np.pad(s0, ((h1, h1), (h2, h2)), mode="edge")
        acc = np.zeros((n1, n2))
        for a in range(s1):
            for b in range(s2):
                acc += p[a:a + n1, b:b + n2]
        s0 = acc / (s1 * s2)
    return 1.0 / s0


def acquisi(nz, nx, dx, dz, zsc, zrc, h_offset, ds, dr, slag, rlag, acq_type="fixspread"):
    """Source/receiver grid indices (1-based, unpadded) of ``SRC/MNAD/acquisi.m:88-190``.

    Returns ``(xs, zs, xr_list, zr_list)``; the reference converts these to
    metres and the driver back to padded indices (``+ d_pml``).
    """
    ds = int(math.trunc(ds / dx)) or 1
    dr = int(math.trunc(dr / dx)) or 1
    xs = np.arange(math.ceil(slag / dx), nx - math.floor(slag / dx) + 1, ds)
    zs = np.zeros_like(xs) + math.floor(zsc / dz)
    h_off = math.floor(h_offset / dx)
    last = nx - math.floor(rlag / dx)
    xr, zr = [], []
    for s in xs:
        if acq_type == "fixspread":
            r = np.arange(math.ceil(rlag / dx), last + 1, dr)
        elif acq_type == "onesided":
            r = np.arange(s, last + 1, dr) if s + h_off > last else np.arange(s, s + h_off, dr)
        elif acq_type == "splitspread":
            if s + h_off > last:
                r = np.arange(s - h_off, last + 1, dr)
            elif s - h_off <= 0:
                r = np.arange(1, s + h_off, dr)
            else:
                r = np.arange(s - h_off, s + h_off, dr)
        else:
            raise ValueError(f"unknown acquisition type {acq_type!r}")
        xr.append(r)
        zr.append(np.zeros_like(r) + math.floor(zrc / dz))
    return xs, zs, xr, zr
