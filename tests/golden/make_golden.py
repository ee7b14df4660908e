"""Generate the golden fixtures of tests/golden/ from the literal restatement.

The reference (MATLAB) cannot run here and ships no golden vectors, so the
fixtures come from oracle/mnad_oracle.py, the sparse-operator restatement of
SRC/MNAD/A??_gen.m, C_cof.m, Ux123_gen.m, Uz123_gen.m, fwd_PDE_exact_MNAD.m
and SRC/migration/Born_adj_MNAD.m.  They pin the oracle and give the GPU
tests reference answers without running the oracle.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import mnad_oracle as P  # noqa: E402


def fwd_small():
    rng = np.random.default_rng(11)
    nz, nx, d = 40, 52, 8
    z = np.arange(nz)[:, None]
    v = np.where(z < 20, 1700.0, 2300.0) + 300.0 * rng.random((nz, nx))
    dx, dz, dt, nt, T = 10.0, 12.5, 1e-3, 180, 3
    w = P.ricker(25.0, dt, nt)
    xr = np.arange(1, nx + 1, 3)
    zr = np.full(xr.size, d + 2)
    zr[0] = 1                 # one receiver in the top strip corner
    zs, xs = d, 14            # source on the last row of the top strip
    steps = np.array([60, 180])
    out = P.fwd_pde_exact_mnad(dx, xs, xr, dz, zs, zr, v, dt, nt, w, d, indx=1, T=T, keep_steps=tuple(steps))
    np.savez_compressed(os.path.join(HERE, "golden_fwd_small.npz"), v=v, dx=dx, dz=dz, dt=dt, nt=nt, d=d, T=T,
                        w=w, xr=xr, zr=zr, zs=zs, xs=xs, steps=steps, datau=out["datau"], UU=out["UU"],
                        illum=out["illum"], fields=np.stack([out["fields"][int(t)][0] for t in steps]),
                        fields_v=np.stack([out["fields"][int(t)][1] for t in steps]),
                        fields_w=np.stack([out["fields"][int(t)][2] for t in steps]), nf=out["nf"])


def rtm_small():
    rng = np.random.default_rng(12)
    nz, nx, d = 44, 60, 8
    z = np.arange(nz)[:, None]
    v = np.where(z < 24, 1800.0, 2500.0) + 100.0 * rng.random((nz, nx))
    vs = np.where(z < 24, 1800.0, 2150.0) + 0.0 * v
    dx, dz, dt, nt = 10.0, 10.0, 1e-3, 220
    w = P.ricker(25.0, dt, nt)
    xr = np.arange(d + 1, nx - d + 1)
    zr = np.full(xr.size, d + 2)
    zs, xs = d + 1, nx // 2
    nf, T = P.snapshot_plan(vs, nt)
    A = P.a_gen(dx, dz, dt, v)
    As = P.a_gen(dx, dz, dt, vs)
    data = P.fwd_pde_exact_mnad(dx, xs, xr, dz, zs, zr, v, dt, nt, w, d, A=A)["datau"]
    bg = P.fwd_pde_exact_mnad(dx, xs, xr, dz, zs, zr, vs, dt, nt, w, d, A=As, indx=1)
    res = data - bg["datau"]
    Im = P.born_adj_mnad(dx, dz, nt, dt, vs, xr, zr, res, d, bg["UU"], A=As)
    np.savez_compressed(os.path.join(HERE, "golden_rtm_small.npz"), v=v, vs=vs, dx=dx, dz=dz, dt=dt, nt=nt, d=d,
                        T=T, nf=nf, w=w, xr=xr, zr=zr, zs=zs, xs=xs, data=res, UU=bg["UU"], illum=bg["illum"],
                        Im=Im, datau=data)


if __name__ == "__main__":
    fwd_small()
    rtm_small()
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))
