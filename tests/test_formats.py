"""The reference drivers' .mat outputs, written by mnad.reference_api.

* data_MNAD_Acoustic.mat (SRC/migration/main_Acoustic_RTM.m:183,
  SRC/modeling/main_Acoustic_Data.m:179): ``data``, a 1 x ns cell whose
  entries are the 1 x 1 cells returned by fwd_PDE_exact_MNAD, and the
  ``profile`` struct;
* data_scattered_MNAD_Acoustic.mat (main_Acoustic_RTM.m:234): ``data_sct``,
  a 1 x ns cell of nt x nr gathers, and ``profile``;
* Illuminations/illum_0.mat (main_Acoustic_RTM.m:244).

Checked by reading the files back with scipy.io as MATLAB's load would see
them: cell nesting, shapes, values, struct fields.
"""
import numpy as np
import scipy.io

from mnad import reference_api as R


def _profile(ns):
    return R.make_profile(fc=15.0, dt=7.5e-4, T_max=3.0, dx=13.0, nx=400, dz=13.0, nz=200, ns=ns)


def _gathers(ns, nt=50, nr=7, seed=0):
    rng = np.random.default_rng(seed)
    return [np.asfortranarray(rng.standard_normal((nt, nr))) for _ in range(ns)]


def test_data_file_round_trip(tmp_path):
    g = _gathers(3)
    path = str(tmp_path / "data_MNAD_Acoustic.mat")
    R.save_data(path, [[x] for x in g], _profile(3))      # the forward's 1 x 1 cells
    m = scipy.io.loadmat(path)
    assert m["data"].shape == (1, 3)                      # data{ss}
    assert m["data"][0, 1].shape == (1, 1)                # data{ss}{1}
    assert np.array_equal(m["data"][0, 1][0, 0], g[1])
    shots, prof = R.load_data(path)
    assert all(np.array_equal(a, b) for a, b in zip(shots, g))
    assert list(prof) == list(R.PROFILE_FIELDS)
    assert prof["f_max"] == 45.0 and prof["ns"] == 3.0


def test_scattered_file_and_illumination(tmp_path):
    g = _gathers(2, seed=1)
    p = str(tmp_path / "data_scattered_MNAD_Acoustic.mat")
    R.save_scattered(p, g, _profile(2))
    m = scipy.io.loadmat(p)
    assert m["data_sct"].shape == (1, 2)
    assert np.array_equal(m["data_sct"][0, 0], g[0])     # data_sct{ss} is the gather itself
    assert m["profile"][0, 0]["dx"][0, 0] == 13.0
    il = np.abs(np.random.default_rng(2).standard_normal((20, 30)))
    q = str(tmp_path / "illum_0.mat")
    R.save_illum_average(q, il)
    assert np.array_equal(scipy.io.loadmat(q)["illum"], il)


def test_writers_refuse_variables_matlab_could_not_read(tmp_path, monkeypatch):
    """MAT v5 keeps at most 2 GiB per variable: a larger one is refused with a
    clear error rather than written into a file MATLAB's load rejects (the
    limit is lowered here so the test needs no 2 GiB array)."""
    import pytest
    monkeypatch.setattr(R, "MAT_V5_MAX_BYTES", 1000)
    g = _gathers(2, nt=50, nr=7)                  # 2 x 2800 bytes
    with pytest.raises(ValueError, match="at most 1000 bytes"):
        R.save_scattered(str(tmp_path / "big.mat"), g, _profile(2))
    R.save_illum_average(str(tmp_path / "small.mat"), np.ones((10, 10)))   # 800 bytes: written
