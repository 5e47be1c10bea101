"""Band-structure mode (src/band_calc.f90:30-92): the kpts reader and the
energy/velocity writers on CPU, and the whole mode through the CUDA library
against the oracle's eigenvalues on a GPU."""
import os

import numpy as np
import pytest

from mepinterp_gb300 import bands, cli, tb_io
from mepinterp_gb300.generator import random_tb_model
from oracle import ref_numpy as O


def test_kpts_file_round_trip(tmp_path):
    kp = bands.k_path([[0, 0, 0], [0.5, 0, 0], [0.5, 0.5, 0], [0, 0, 0]], 7)
    assert kp.shape == (22, 3)
    p = tmp_path / "kpts"
    bands.write_kpts_file(str(p), kp)
    assert np.allclose(bands.read_kpts_file(str(p)), kp, atol=1e-10)


def test_energy_writers(tmp_path):
    rng = np.random.default_rng(0)
    kp = rng.uniform(-0.5, 0.5, (5, 3))
    E = np.sort(rng.normal(size=(5, 4)), axis=1)
    raw = tmp_path / "raw"
    raw.mkdir()
    for i, e in enumerate(E, start=1):
        bands.write_en_binary(str(raw), i, e)
    assert (raw / "enK.0000003").stat().st_size == 4 * 8
    assert np.array_equal(bands.read_en_binary(str(raw), 3), E[2])
    path = bands.write_en_global(str(tmp_path), kp, E)
    idx, k, e = bands.read_en_global(path)
    assert np.array_equal(idx, np.repeat(np.arange(1, 6), 4))
    assert np.allclose(k, np.repeat(kp, 4, axis=0), atol=1e-8)
    assert np.allclose(e, E.ravel(), atol=1e-8)
    V = rng.normal(size=(3, 4, 4)) + 1j * rng.normal(size=(3, 4, 4))
    vp = bands.write_velo(str(tmp_path), 2, V)
    rows = [l.split() for l in open(vp) if not l.strip().startswith("#")]
    assert len(rows) == 3 * 16
    x, n, m, re, im = (float(v) for v in rows[5])   # x = 1, m = 2, n = 2 (n fastest)
    assert (x, n, m) == (1, 2, 2) and abs(re - V[0, 1, 1].real) < 1e-7 and abs(im - V[0, 1, 1].imag) < 1e-7


@pytest.mark.gpu
def test_band_mode_cli(gpu_lib, tmp_path):
    m = random_tb_model(n_wf=8, r_max=1, seed=4)
    w90 = tmp_path / "w90files"
    w90.mkdir()
    tb_io.write_hr_file(str(w90 / "wf1_hr.dat"), m)
    tb_io.write_r_file(str(w90 / "wf1_r.dat"), m)
    tb_io.write_input_cfg(str(tmp_path / "input.cfg"), seed_name="wf1", a_latt=m.a_latt, mp_grid=(4, 4, 4),
                          valence_bands=4, wf_centers=m.wf_centers, plot_bands=True, do_write_velo=True)
    kp = bands.k_path([[0, 0, 0], [0.5, 0, 0], [0.5, 0.5, 0.5]], 10)
    bands.write_kpts_file(str(tmp_path / "kpts"), kp)
    assert cli.main([str(tmp_path)]) == 0
    back = tb_io.read_tb_basis(str(w90), "wf1", wf_centers=m.wf_centers, a_latt=m.a_latt)
    E_ref = O.interp_k(back.as_dict(), kp)[0]
    raw = np.stack([bands.read_en_binary(str(tmp_path / "raw"), i + 1) for i in range(kp.shape[0])])
    assert np.abs(raw - E_ref).max() <= 1e-10 * np.abs(E_ref).max()
    idx, k, e = bands.read_en_global(str(tmp_path / "out" / "eBands.dat"))   # printed as f18.8
    assert np.abs(e.reshape(E_ref.shape) - E_ref).max() <= 1e-8
    assert len(os.listdir(tmp_path / "out" / "velo")) == kp.shape[0]
