"""The ./Wavefields hand-off of the reference through files.

fwd_PDE_exact_MNAD with indx = 1 saves Wavefields/UU_<ss>.mat and
Illuminations/illum_<ss>.mat (SRC/MNAD/fwd_PDE_exact_MNAD.m:160-164), and
Born_adj_MNAD loads UU_<ss>.mat (SRC/migration/Born_adj_MNAD.m:33) -- in the
reference's parfor the two may run in different worker processes.  Here the
forward runs in one context, its stored wavefield is written with
save_wavefield, and a second context (another process's library state) loads
it with load_wavefield and runs the adjoint.  FP32 snapshots survive the
FP64 file exactly, so the image equals the one imaged from device storage bit
for bit; the files hold the reference's variables and shapes.
"""
import numpy as np
import pytest
import scipy.io

import mnad
from mnad import reference_api as R
from mnad import workflow

pytestmark = pytest.mark.gpu


def test_born_adj_from_a_reloaded_wavefield_file(tmp_path):
    from mnad import build
    build.build()
    nz, nx, d, nt, T = 90, 120, 15, 300, 4
    rng = np.random.default_rng(3)
    z = np.arange(nz)[:, None]
    v = np.asfortranarray(np.where(z < 45, 1800.0, 2400.0) + 60.0 * rng.random((nz, nx)))
    vs = np.asfortranarray(np.full((nz, nx), 1900.0))
    w = workflow.ricker(25.0, 1e-3, nt)
    xr = np.arange(d + 1, nx - d + 1, dtype=float)
    zr = np.full(xr.size, d + 2.0)
    args = (10.0, float(nx // 2), xr, 10.0, float(d + 1), zr)
    ss = 5
    with mnad.Context(0, T=T) as a:
        data = R.fwd_PDE_exact_MNAD(*args, v, 1e-3, nt, w, d, ss, ctx=a)
        datas = R.fwd_PDE_exact_MNAD(*args, vs, 1e-3, nt, w, d, ss, indx=1, ctx=a)
        sct = data[0] - datas[0]
        im_device = R.Born_adj_MNAD(10.0, 10.0, nt, 1e-3, vs, xr, zr, sct, d, ss, ctx=a)
        UU_dev, illum_dev = a.wavefield_export(ss)
        R.save_wavefield(a, ss, nz, nx, d, directory=str(tmp_path))
    UU = scipy.io.loadmat(str(tmp_path / "Wavefields" / f"UU_{ss}.mat"))["UU"]
    illum = scipy.io.loadmat(str(tmp_path / "Illuminations" / f"illum_{ss}.mat"))["illum"]
    assert np.array_equal(UU, UU_dev)
    assert illum.shape == (nz - 2 * d, nx - 2 * d)
    assert np.array_equal(illum.ravel(order="F"), illum_dev)
    with mnad.Context(0, T=T) as b:            # a fresh library state: only the files connect the two
        R.load_wavefield(b, ss, nz, nx, d, nt, T, directory=str(tmp_path))
        info = b.wavefield_info(ss)
        assert info["ncols"] == UU.shape[1] and info["nsnap"] == nt // T
        im_file = R.Born_adj_MNAD(10.0, 10.0, nt, 1e-3, vs, xr, zr, [sct], d, ss, ctx=b)
    assert im_file.shape == ((nz - 2 * d) * (nx - 2 * d), 1)
    assert np.linalg.norm(im_device) > 0
    assert np.array_equal(im_file, im_device)
