"""CPU tests of the FP64 oracle (no GPU).

The oracle is two independent restatements of the reference MATLAB code:
the literal sparse-operator one (oracle/mnad_oracle.py) and the matrix-free
C one (oracle/mnad_oracle.c).  They must agree to FP64 rounding, match the
structural facts of the generator files, follow the reference's step order,
and reproduce the committed golden fixtures.
"""
import math
import os

import numpy as np
import pytest

from oracle import coracle
from oracle import mnad_oracle as P

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


@pytest.fixture(scope="module")
def small():
    rng = np.random.default_rng(3)
    nz, nx, d = 26, 33, 6
    v = 1500 + 1000 * rng.random((nz, nx))
    return dict(v=v, dx=10.0, dz=12.0, dt=1e-3, d=d, nt=120,
                xr=np.array([1, 4, 9, 17, 33, 33]), zr=np.array([2, 7, 7, 1, 26, 26]),
                zs=3, xs=5)   # source inside the top CPML strip


def test_operator_nnz_and_offsets():
    """63 nonzeros per interior row: 9+8+8+6+9+4+6+4+9 (A??_gen.m)."""
    nz, nx = 17, 19
    v = np.full((nz, nx), 2000.0)
    A = P.a_gen(10.0, 10.0, 1e-3, v)
    per = {"Auu": 9, "Auv": 8, "Auw": 8, "Avu": 6, "Avv": 9, "Avw": 4, "Awu": 6, "Awv": 4, "Aww": 9}
    row = 8 + 9 * nz   # interior point (j=8, i=9), 0-based
    for k, n in per.items():
        assert A[k][row].nnz == n, k
    assert sum(A[k][row].nnz for k in per) == 63
    # Auv couples V at x+-1, x+-2 and the diagonals only: no z-only offsets.
    cols = sorted(A["Auv"][row].indices - row)
    assert cols == sorted([-2 * nz, -nz - 1, -nz, -nz + 1, nz - 1, nz, nz + 1, 2 * nz])
    cols = sorted(A["Auw"][row].indices - row)
    assert cols == sorted([-2, -nz - 1, -1, nz - 1, -nz + 1, 1, nz + 1, 2])


def test_operator_antisymmetry():
    """Auv is odd in x and Auw odd in z (Auv_gen.m:29/128, Auw_gen.m:29/212)."""
    nz, nx = 15, 15
    v = np.full((nz, nx), 2300.0)
    A = P.a_gen(8.0, 11.0, 1e-3, v)
    row = 7 + 7 * nz
    auv = A["Auv"][row].toarray().ravel()
    auw = A["Auw"][row].toarray().ravel()
    for off in (nz, 2 * nz, nz + 1, nz - 1):
        assert auv[row + off] == pytest.approx(-auv[row - off], rel=1e-14)
    for off in (1, 2, nz + 1, 1 - nz):
        assert auw[row + off] == pytest.approx(-auw[row - off], rel=1e-14)


def test_out_of_grid_neighbours_are_omitted():
    """Boundary rows lose the entries whose neighbour falls outside the grid."""
    nz, nx = 9, 11
    A = P.a_gen(10.0, 10.0, 1e-3, np.full((nz, nx), 2000.0))
    corner = 0
    assert A["Auu"][corner].nnz == 4      # centre, z+1, x+1, (z+1,x+1)
    assert A["Auv"][corner].nnz == 3      # x+1, (z+1,x+1), x+2
    assert A["Avw"][corner].nnz == 1


def test_cpml_coefficients_are_strip_only():
    nz, nx, d = 30, 40, 7
    v = np.full((nz, nx), 2500.0)
    c = P.c_cof(1e-4, d, 10.0, 12.0, 1e-3, nx, nz, v)
    assert np.all(c["c1xl"][:, d:] == 1) and np.all(c["c2xl"][:, d:] == 0) and np.all(c["c3xl"][:, d:] == 0)
    assert np.all(c["c1xr"][:, :nx - d] == 1) and np.all(c["c3xr"][:, :nx - d] == 0)
    assert np.all(c["c1zt"][d:, :] == 1) and np.all(c["c1zb"][:nz - d, :] == 1)
    assert np.all(c["c3xl"][:, :d] > 0) and np.all(c["c3zb"][nz - d:, :] > 0)
    # damping grows towards the outer edge (X = D, D-h, ..., h)
    assert np.all(np.diff(c["c3xl"][0, :d]) < 0) and np.all(np.diff(c["c3xr"][0, nx - d:]) > 0)


def test_snapshot_plan_formula():
    v = np.array([[1500.0, 3500.0]])
    nf = P.snapshot_nf(v, 3000)
    assert nf == math.floor(3000 / (6 * 3500 / 1500))
    assert P.snapshot_plan(v, 3000) == (nf, math.floor(3000 / nf / 2))
    with pytest.raises(ZeroDivisionError):
        P.snapshot_plan(np.array([[1500.0, 4500.0]]), 10)


def test_sparse_and_matrix_free_oracles_agree(small):
    s = small
    w = P.ricker(25.0, s["dt"], s["nt"])
    T = 3
    nf = P.snapshot_nf(s["v"], s["nt"])
    po = P.fwd_pde_exact_mnad(s["dx"], s["xs"], s["xr"], s["dz"], s["zs"], s["zr"], s["v"], s["dt"], s["nt"], w,
                              s["d"], indx=1, T=T, record_vw=True, keep_steps=(40, 120))
    co = coracle.fwd(s["dx"], s["xs"], s["xr"], s["dz"], s["zs"], s["zr"], s["v"], s["dt"], s["nt"], w, s["d"],
                     indx=1, T=T, ncols=po["UU"].shape[1], record_vw=True, keep_steps=(40, 120))
    assert po["UU"].shape[1] == max(2 * nf + 1, s["nt"] // T)
    for k in ("datau", "datav", "dataw", "UU", "illum"):
        assert rel(co[k], po[k]) < 1e-12, k
    for t in (40, 120):
        for f in range(3):
            assert rel(co["fields"][t][f], po["fields"][t][f]) < 1e-12
    Ip = P.born_adj_mnad(s["dx"], s["dz"], s["nt"], s["dt"], s["v"], s["xr"], s["zr"], [po["datau"]], s["d"],
                         po["UU"], T=T)
    Ic = coracle.adj(s["dx"], s["dz"], s["nt"], s["dt"], s["v"], s["xr"], s["zr"], po["datau"], s["d"], po["UU"], T)
    assert rel(Ic, Ip) < 1e-12
    Ia = P.born_adj_mnad(s["dx"], s["dz"], s["nt"], s["dt"], s["v"], s["xr"], s["zr"], po["datau"], s["d"],
                         po["UU"], T=T, pairing="aligned")
    Ica = coracle.adj(s["dx"], s["dz"], s["nt"], s["dt"], s["v"], s["xr"], s["zr"], po["datau"], s["d"], po["UU"], T,
                      pairing="aligned")
    assert rel(Ica, Ia) < 1e-12


def test_source_is_injected_after_the_cpml_update(small):
    """fwd_PDE_exact_MNAD.m:95-111: CPML memory first, then the injection.

    With the source inside a strip, injecting before the CPML update changes
    the result; the oracle must not."""
    s = small
    w = P.ricker(25.0, s["dt"], 40)
    ref = P.fwd_pde_exact_mnad(s["dx"], s["xs"], s["xr"], s["dz"], s["zs"], s["zr"], s["v"], s["dt"], 40, w, s["d"])
    # same loop with the injection moved in front of the CPML update
    v = s["v"]
    nz, nx = v.shape
    A = P.a_gen(s["dx"], s["dz"], s["dt"], v)
    c = P.c_cof(1e-4, s["d"], s["dx"], s["dz"], s["dt"], nx, nz, v)
    r = v**2 * s["dt"]**2
    F = [np.zeros((nz, nx)) for _ in range(6)]
    M = [P._new_mem(nz, nx) for _ in range(3)]
    pU, U, pV, V, pW, W = F
    out = np.zeros(40)
    for tt in range(1, 41):
        U[s["zs"] - 1, s["xs"] - 1] += r[s["zs"] - 1, s["xs"] - 1] * w[tt - 1]
        cu = P.ux123_gen(M[0], U, s["dx"], c) + P.uz123_gen(M[0], U, s["dz"], c)
        cv = P.ux123_gen(M[1], V, s["dx"], c) + P.uz123_gen(M[1], V, s["dz"], c)
        cw = P.ux123_gen(M[2], W, s["dx"], c) + P.uz123_gen(M[2], W, s["dz"], c)
        nU = P._apply(A["Auu"], U) + P._apply(A["Auv"], V) + P._apply(A["Auw"], W) - pU - r * cu
        nV = P._apply(A["Avv"], V) + P._apply(A["Avu"], U) + P._apply(A["Avw"], W) - pV - r * cv
        nW = P._apply(A["Aww"], W) + P._apply(A["Awu"], U) + P._apply(A["Awv"], V) - pW - r * cw
        out[tt - 1] = U[s["zr"][1] - 1, s["xr"][1] - 1]
        pU, U, pV, V, pW, W = U, nU, V, nV, W, nW
    assert rel(out, ref["datau"][:, 1]) > 1e-6


def test_receivers_sample_post_injection_field():
    """datau(tt) is read from U after this step's injection (:111 then :120)."""
    nz, nx, d = 20, 20, 4
    v = np.full((nz, nx), 2000.0)
    w = np.zeros(5)
    w[0] = 1.0
    out = P.fwd_pde_exact_mnad(10.0, 10, [10], 10.0, 10, [10], v, 1e-3, 5, w, d)
    assert out["datau"][0, 0] == pytest.approx(2000.0**2 * 1e-6)


def test_adjoint_injects_after_the_update():
    """Born_adj_MNAD.m:109-111: the residual of step tt enters U after nU is
    formed, so it only reaches the field through -pU one step later."""
    nz, nx, d = 20, 20, 4
    v = np.full((nz, nx), 2000.0)
    nt, T = 6, 1
    data = np.zeros((nt, 1))
    data[nt - 1, 0] = 1.0
    UU = np.zeros(((nz - 2 * d) * (nx - 2 * d), nt))
    UU[:, :] = 1.0
    Im = P.born_adj_mnad(10.0, 10.0, nt, 1e-3, v, [10], [10], data, d, UU, T=T)
    # After step nt the new U is zero everywhere (injection not yet felt) ...
    # ... after step nt-1 the field is -r*data at the receiver only.
    r = (2000.0 * 1e-3) ** 2
    q = (10 - 1 - d) + (10 - 1 - d) * (nz - 2 * d)
    assert abs(Im).sum() > 0
    Im1 = P.born_adj_mnad(10.0, 10.0, 2, 1e-3, v, [10], [10], data[-2:], d, UU[:, :2], T=1)
    assert Im1[q] == pytest.approx(-r)
    assert np.count_nonzero(Im1) == 1


def test_reference_pairing_shifts_when_columns_exceed_k():
    """D3: ncols = 2nf+1 > k shifts the pairing by (ncols-k)*T steps."""
    nz, nx, d = 16, 16, 3
    nint = (nz - 2 * d) * (nx - 2 * d)
    nt, T = 12, 3                           # k = 4 snapshots
    UU = np.zeros((nint, 5))                # ncols = 5 > k: last column zero
    UU[:, :4] = np.arange(1, 5)[None, :]
    v = np.full((nz, nx), 2000.0)
    data = np.random.default_rng(0).standard_normal((nt, 2))
    ref = P.born_adj_mnad(10.0, 10.0, nt, 1e-3, v, [5, 9], [6, 6], data, d, UU, T=T)
    ali = P.born_adj_mnad(10.0, 10.0, nt, 1e-3, v, [5, 9], [6, 6], data, d, UU[:, :4], T=T, pairing="aligned")
    assert rel(ref, ali) > 1e-3
    same = P.born_adj_mnad(10.0, 10.0, nt, 1e-3, v, [5, 9], [6, 6], data, d, UU[:, :4], T=T)
    assert rel(same, ali) < 1e-15         # ncols == k: reference pairing is aligned


@pytest.mark.parametrize("name", ["golden_fwd_small", "golden_rtm_small"])
def test_oracle_reproduces_golden_fixture(name):
    path = os.path.join(GOLDEN, name + ".npz")
    g = np.load(path)
    if name == "golden_fwd_small":
        out = coracle.fwd(float(g["dx"]), int(g["xs"]), g["xr"], float(g["dz"]), int(g["zs"]), g["zr"], g["v"],
                          float(g["dt"]), int(g["nt"]), g["w"], int(g["d"]), indx=1, T=int(g["T"]),
                          ncols=g["UU"].shape[1], keep_steps=tuple(int(t) for t in g["steps"]))
        assert rel(out["datau"], g["datau"]) < 1e-12
        assert rel(out["UU"], g["UU"]) < 1e-12
        assert rel(out["illum"], g["illum"]) < 1e-12
        for k, t in enumerate(g["steps"]):
            assert rel(out["fields"][int(t)][0], g["fields"][k]) < 1e-12
    else:
        Im = coracle.adj(float(g["dx"]), float(g["dz"]), int(g["nt"]), float(g["dt"]), g["vs"], g["xr"], g["zr"],
                         g["data"], int(g["d"]), g["UU"], int(g["T"]))
        assert rel(Im, g["Im"]) < 1e-12
