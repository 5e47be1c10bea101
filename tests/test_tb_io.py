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
    g = np.load(GOLD)
    H = g["H_eV_0p900"]
    R = g["R_0p900"]
    # write the fixture in the reference's layout (R, m fastest inside, m n Re Im)
    p = tmp_path / "FeMn_hr.dat"
    with open(p, "w") as f:
        f.write("FeMn\n8\n27\n")
        f.write(" ".join(["1"] * 15) + "\n" + " ".join(["1"] * 12) + "\n")
        for r in range(27):
            for n in range(8):
                for m in range(8):
                    f.write(f"{R[r,0]} {R[r,1]} {R[r,2]} {m+1} {n+1} {H[r,m,n].real:.6f} {H[r,m,n].imag:.6f}\n")
    Rb, Hb, deg = tb_io.read_hr_file(str(p))
    assert deg.size == 27
    assert np.allclose(Rb, R)
    assert np.abs(Hb * AU_TO_EV - H).max() < 1e-6


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
