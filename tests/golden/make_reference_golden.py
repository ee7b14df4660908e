"""Golden fixtures produced by the reference's own MATLAB sources.

Runs SRC/MNAD/*.m and SRC/migration/Born_adj_MNAD.m of a reference checkout
(its path is the first argument, or MNAD_REFERENCE) under the MATLAB-
subset interpreter oracle/mlite.py -- neither MATLAB nor Octave exists here --
and stores their outputs:

* golden_ref_rtm.npz: one RTM shot on a 40 x 52 layered model (true-model
  forward, background forward with indx = 1 -> UU and illum, adjoint of the
  scattered data -> Im) at three record lengths: nt = 240, where
  floor(nt/T) < 2nf+1 (the reference's pairing shifted by one snapshot),
  nt = 247 (aligned) and nt = 239, where floor(nt/T) > 2nf+1 and UU grows
  past its preallocated columns;
* golden_ref_constant_velocity.npz: the constant-velocity shot (201 x 201, 20-point CPML, 2000 m/s,
  20 Hz Ricker at the centre, 201 receivers on row 21, nt = 1000), the
  reference's own CPU case;
* golden_ref_prep.npz: SRC/MNAD/acquisi.m for the 'fixspread', 'onesided',
  'splitspread' and 'obn' geometries and SRC/MNAD/v_smooth.m on a random
  model (the drivers' acquisition and migration-model preparation).

The only change applied to the reference sources is the one-token fix of
Born_adj_MNAD.m:105-106 (undefined U_r read as U); the adjoint receives the
data as a cell {data}, as Born_adj_MNAD.m:50 expects.  The Ricker wavelet of
the drivers (main_Acoustic_RTM.m:138-140) is an input, computed here.

Usage: python tests/golden/make_reference_golden.py <reference checkout>
   or: MNAD_REFERENCE=<reference checkout> python tests/golden/make_reference_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "mnad-modeling-rtm_gb300"))

from oracle import mlite  # noqa: E402

REF = None   # the reference checkout, set by main()
NAMES = ["Auu", "Auv", "Auw", "Avu", "Avv", "Avw", "Awu", "Awv", "Aww"]


def S(x):
    return np.array([[float(x)]])


def ricker(fc, dt, nt):
    t = np.arange(nt) * dt
    tau = np.pi * (t - 1.1 / fc) * fc
    return ((1 - 2 * tau ** 2) * np.exp(-tau ** 2)).reshape(-1, 1)


def interpreter():
    return mlite.Interpreter([os.path.join(REF, "SRC", "MNAD"), os.path.join(REF, "SRC", "migration")],
                             patches={"Born_adj_MNAD": [("U_r(:)", "U(:)")]})


def operators(it, dx, dz, dt, v):
    return [it.call(n + "_gen", [S(dx), S(dz), S(dt), v])[0] for n in NAMES]


def rtm_case(it, nt, seed=0):
    nz, nx, d = 40, 52, 8
    dx = dz = 10.0
    dt = 1e-3
    z = np.arange(nz)[:, None] * np.ones((1, nx))
    x = np.ones((nz, 1)) * np.arange(nx)[None, :]
    v = 1700.0 + 600.0 * (z >= 20) + 500.0 * (z >= 30)
    v = v + 250.0 * np.exp(-((z - 25) ** 2 + (x - 30) ** 2) / (2 * 4.0 ** 2))
    vs = 1700.0 + 1100.0 * (z / (nz - 1)) + 0.0 * x          # smooth background
    w = ricker(25.0, dt, nt)
    xr = np.arange(d + 1, nx - d + 1, dtype=float).reshape(1, -1)
    zr = np.full(xr.shape, d + 2.0)
    zs, xs, ss = d + 2, 27, 5
    A = operators(it, dx, dz, dt, v)
    As = operators(it, dx, dz, dt, vs)
    common = [S(dx), S(xs), xr, S(dz), S(zs), zr]
    data = it.call("fwd_PDE_exact_MNAD", common + [v, S(dt), S(nt), w, S(d), S(ss)] + A + [S(0)])[0].items[0]
    datas = it.call("fwd_PDE_exact_MNAD", common + [vs, S(dt), S(nt), w, S(d), S(ss)] + As + [S(1)])[0].items[0]
    UU = it.files[f"./Wavefields/UU_{ss}"]["UU"]
    illum = it.files[f"./Illuminations/illum_{ss}"]["illum"]
    res = data - datas
    Im = it.call("Born_adj_MNAD", [S(dx), S(dz), S(nt), S(dt), vs, xr, zr, mlite.Cell([res]), S(d), S(ss)] + As)[0]
    return dict(v=v, vs=vs, dx=dx, dz=dz, dt=dt, nt=nt, d=d, w=w.ravel(), xr=xr.ravel(), zr=zr.ravel(), zs=zs,
                xs=xs, data=data, datas=datas, UU=UU, illum=illum, Im=Im.ravel())


def constant_velocity_case(it):
    nz = nx = 201
    d, nt, dt, dx = 20, 1000, 1e-3, 10.0
    v = np.full((nz, nx), 2000.0)
    w = ricker(20.0, dt, nt)
    xr = np.arange(1, nx + 1, dtype=float).reshape(1, -1)
    zr = np.full(xr.shape, 21.0)
    A = operators(it, dx, dx, dt, v)
    data = it.call("fwd_PDE_exact_MNAD", [S(dx), S(101), xr, S(dx), S(101), zr, v, S(dt), S(nt), w, S(d), S(1)] +
                   A + [S(0)])[0].items[0]
    return dict(dx=dx, dt=dt, nt=nt, d=d, v0=2000.0, nz=nz, nx=nx, zs=101, xs=101, zr=21, fc=20.0, data=data)


ACQ = dict(dx=10.0, dz=10.0, zsc=20.0, zrc=20.0, h_offset=500.0, ds=100.0, dr=20.0, slag=50.0, rlag=30.0)


def prep_case(it):
    rng = np.random.default_rng(3)
    V = np.full((60, 200), 2400.0)
    V[:7, :] = 1500.0                                  # water column for the 'obn' geometry
    V[7:, 80:] += 300.0
    out = dict(V=V, **{f"acq_{k}": v for k, v in ACQ.items()})
    a = ACQ
    for kind in ("fixspread", "onesided", "splitspread", "obn"):
        Src, Rec = it.call("acquisi", [V, S(a["dx"]), S(a["dz"]), S(a["zsc"]), S(a["zrc"]), S(a["h_offset"]),
                                       S(a["ds"]), S(a["dr"]), S(a["slag"]), S(a["rlag"]), kind,
                                       np.zeros((1, 1)) == 1], 2)
        ns = Src.shape[1]
        xr = [Rec.items[2 * k].ravel() for k in range(ns)]
        zr = [Rec.items[2 * k + 1].ravel() for k in range(ns)]
        out[f"{kind}_Source"] = Src
        out[f"{kind}_xr"] = np.concatenate(xr)
        out[f"{kind}_zr"] = np.concatenate(zr)
        out[f"{kind}_nr"] = np.array([len(x) for x in xr])
    vm = rng.uniform(1500.0, 3500.0, (24, 30))
    out["vsm_in"] = vm
    out["vsm_out"] = it.call("v_smooth", [vm, S(5), S(3), S(2)])[0]
    return out


def main():
    it = interpreter()
    cases = {"a": rtm_case(it, 240), "b": rtm_case(it, 247), "c": rtm_case(it, 239)}
    out = {f"{n}_{k}": val for n, case in cases.items() for k, val in case.items()}
    np.savez_compressed(os.path.join(HERE, "golden_ref_rtm.npz"), **out)
    np.savez_compressed(os.path.join(HERE, "golden_ref_prep.npz"), **prep_case(it))
    c = constant_velocity_case(it)
    np.savez_compressed(os.path.join(HERE, "golden_ref_constant_velocity.npz"), **c)
    for name, case in cases.items():
        print(name, "nt", case["nt"], "UU", case["UU"].shape, "|Im|", np.linalg.norm(case["Im"]))
    print("constant velocity |data|", np.linalg.norm(c["data"]))


def reference_path():
    path = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MNAD_REFERENCE")
    if not path or not os.path.isdir(os.path.join(path, "SRC", "MNAD")):
        sys.exit("usage: make_reference_golden.py <reference checkout>  (or set MNAD_REFERENCE); "
                 "the checkout must contain SRC/MNAD and SRC/migration")
    return path


if __name__ == "__main__":
    REF = reference_path()
    main()
