"""CPU tests of the reference-format readers/writers and the output stage."""
import os

import numpy as np
import pytest

from mepinterp_gb300 import output, tb_io
from mepinterp_gb300.generator import AU_TO_EV, random_tb_model
from oracle import ref_numpy as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "femn.npz")


def test_hr_r_round_trip(tmp_path):
    m = random_tb_model(n_wf=6, r_max=1, seed=3)
    tb_io.write_hr_file(str(tmp_path / "wf1_hr.dat"), m)
    tb_io.write_r_file(str(tmp_path / "wf1_r.dat"), m)
    back = tb_io.read_tb_basis(str(tmp_path), "wf1", wf_centers=m.wf_centers, a_latt=m.a_latt)
    assert np.array_equal(back.R_frac, m.R_frac)
    # |x| < 1e-7 eV is zeroed on reading (src/file_io.f90:732-733)
    assert np.abs(back.H - m.H).max() <= 1e-7 / AU_TO_EV + 1e-12 * np.abs(m.H).max()
    assert np.abs(back.r - m.r).max() <= 1e-12 * np.abs(m.r).max()


def test_hr_reads_femn_layout(tmp_path):
    """The reader on the reference's own FeMn_hr.dat (delta = 0.9), byte for
    byte as shipped in config/FeMn_TB/delta0.900/w90files/: 8 Wannier
    functions, 27 R vectors, H(R) equal to the fixture's independent parse."""
    g = np.load(GOLD)
    p = tmp_path / "FeMn_hr.dat"
    p.write_bytes(g["hr_dat_0p900"].tobytes())
    Rb, Hb, deg = tb_io.read_hr_file(str(p))
    assert deg.size == 27 and np.all(deg == 1)
    assert np.array_equal(Rb, g["R_0p900"].astype(float))
    assert np.abs(Hb * AU_TO_EV - g["H_eV_0p900"]).max() < 1e-12
    # Hermitian model: H(-R) = H(R)^dag
    idx = {tuple(r): i for i, r in enumerate(Rb.astype(int))}
    for i, r in enumerate(Rb.astype(int)):
        j = idx[tuple(-r)]
        assert np.abs(Hb[j] - Hb[i].conj().T).max() < 1e-12


def test_hr_warns_on_new_r_inside_block(tmp_path):
    """An R vector that changes inside its block is a warning in the reference
    (src/file_io.f90:720-727): the block keeps its first R and the element is
    still stored."""
    m = random_tb_model(n_wf=2, r_max=1, seed=2)
    tb_io.write_hr_file(str(tmp_path / "x_hr.dat"), m)
    lines = (tmp_path / "x_hr.dat").read_text().split("\n")
    # second matrix line of the first R block: give it another R
    first = next(i for i, ln in enumerate(lines) if len(ln.split()) == 7)
    parts = lines[first + 1].split()
    parts[0] = str(int(parts[0]) + 5)
    lines[first + 1] = " ".join(parts)
    (tmp_path / "x_hr.dat").write_text("\n".join(lines))
    with pytest.warns(RuntimeWarning, match="unexpected new R_vect"):
        R, H, _ = tb_io.read_hr_file(str(tmp_path / "x_hr.dat"))
    assert np.array_equal(R, m.R_frac)
    assert np.abs(H - m.H).max() <= 1e-7 / AU_TO_EV + 1e-12 * np.abs(m.H).max()


def test_r_file_order_mismatch(tmp_path):
    m = random_tb_model(n_wf=4, r_max=1, seed=1)
    tb_io.write_r_file(str(tmp_path / "x_r.dat"), m)
    with pytest.raises(tb_io.TBFormatError):
        tb_io.read_r_file(str(tmp_path / "x_r.dat"), m.R_frac[::-1].copy())


def test_input_cfg_round_trip(tmp_path):
    tau = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0]])
    a = np.array([[5.6, 0.0, 3.9], [-2.8, 4.8, 3.9], [-2.8, -4.8, 3.9]])
    tb_io.write_input_cfg(str(tmp_path / "input.cfg"), seed_name="FeMn", a_latt=a, mp_grid=(8, 8, 8),
                          valence_bands=4, wf_centers=tau, eF_min=-1.0, eF_max=1.0, N_eF=5, Tkelvin=300.0)
    cfg = tb_io.read_input_cfg(str(tmp_path / "input.cfg"))
    assert cfg["seed_name"] == "FeMn"
    assert np.allclose(cfg["a_latt"], a)
    assert np.allclose(cfg["wf_centers"], tau)
    assert cfg["mp_grid"] == (8, 8, 8)
    assert np.allclose(cfg["ef_lst"] * AU_TO_EV, np.linspace(-1, 1, 5))
    assert cfg["valence_bands"] == 4 and cfg["T_kelvin"] == 300.0
    assert cfg["do_ahc"] and cfg["do_mep"] and cfg["do_kubo"] and cfg["do_gauge_trafo"]


def test_output_stage_matches_oracle(tmp_path):
    m = random_tb_model(n_wf=8, r_max=1, seed=2).as_dict()
    job = dict(mp_grid=(3, 3, 3), ef_lst=np.linspace(-0.05, 0.05, 7), T_kelvin=0.0, valence_bands=4)
    loc = O.run(m, job)
    a = output.integrate_over_k_space(loc, job["mp_grid"], m["a_latt"], 4)
    b = O.integrate(loc, job["mp_grid"], m["a_latt"], 4)
    assert a["eF_idx"] == b["eF_idx"]
    for k in ("ahc_tens", "mep_ic", "mep_lc", "mep_cs", "mep_tens", "mep_bands", "kubo_mep_tens"):
        assert np.allclose(a[k], b[k], rtol=1e-14, atol=0), k
    files = output.write_outputs(str(tmp_path / "out"), a, job["ef_lst"])
    names = {os.path.basename(f) for f in files}
    assert {"ahc_tens.npy", "mep_tens.npy", "mep_bands.npy", "kubo_mep_tens.npy"} <= names
    x = np.load(tmp_path / "out" / "ahc_tens.npy")
    assert x.flags.f_contiguous and np.allclose(x, a["ahc_tens"])
    assert os.path.exists(tmp_path / "out" / "occ.dat")


def test_fermi_selector_first_minimum():
    assert output.fermi_selector(2, [6.0, 8.0, 8.0, 10.0], 4) == 1
    assert output.fermi_selector(1, [3.0, 5.0], 4) == 0
