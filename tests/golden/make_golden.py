"""Build tests/golden/femn.npz from the reference's FeMn fixtures.

Run in a checkout that has the reference next to it:

    python tests/golden/make_golden.py <path to the reference checkout>

The reference ships, for the FeMn 3Q tight-binding model at strains
delta = 0.9 / 1.0 / 1.1 (config/FeMn_TB/delta*/):

* ``w90files/FeMn_hr.dat``  H(R), 8 Wannier functions, 27 integer R (eV)
* ``FeMn_d*.latt``          the lattice (3 rows = a1, a2, a3, bohr)
* ``ahc_tens.npy``          sigma_ab (3x3, atomic units) from kubo_ahc_tens
* ``ahcVELO_sol*.npy``      velo_ahc_tens over 121 photon energies (3x3x121)

The delta = 0.9 ``FeMn_hr.dat`` is also kept byte for byte (``hr_dat_0p900``,
uint8), so the package's reader is tested on the reference's own file.

The wf centres, N_val = 4, E_F = 0, T = 0, kuboTol = 1e-5 and eta = 0.1 eV are the
ones tests/test_FeMn_AHE.f90:127-217 writes into input.cfg.  The file is parsed
with plain numpy here (not with the package's reader) so the fixture does not
depend on the code it checks.
"""
import os
import sys

import numpy as np


def _parse_hr(path):
    with open(path) as fh:
        lines = fh.read().split("\n")
    n_wf = int(lines[1].split()[0])
    n_r = int(lines[2].split()[0])
    n_deg_lines = (n_r + 14) // 15
    body = np.loadtxt(lines[3 + n_deg_lines:]).reshape(n_r, n_wf * n_wf, 7)
    R = body[:, 0, :3].astype(np.int64)
    H = np.zeros((n_r, n_wf, n_wf), np.complex128)
    for r in range(n_r):
        m = body[r, :, 3].astype(int) - 1
        n = body[r, :, 4].astype(int) - 1
        H[r, m, n] = body[r, :, 5] + 1j * body[r, :, 6]
    return R, H


def main(ref_root):
    out = {}
    tau = np.zeros((8, 3))
    tau[:4, 0] = [0.0, 0.5, 0.5, 0.0]
    tau[:4, 1] = [0.0, 0.5, 0.0, 0.0]
    tau[:4, 2] = [0.0, 0.0, 0.5, 0.5]
    tau[4:] = tau[:4]
    out["wf_centers"] = tau
    for tag in ("0.900", "1.000", "1.100"):
        base = os.path.join(ref_root, "config", "FeMn_TB", "delta" + tag)
        R, H = _parse_hr(os.path.join(base, "w90files", "FeMn_hr.dat"))
        latt_name = [f for f in os.listdir(base) if f.endswith(".latt")][0]
        velo_name = [f for f in os.listdir(base) if f.startswith("ahcVELO")][0]
        key = tag.replace(".", "p")
        out["R_" + key] = R
        out["H_eV_" + key] = H
        out["latt_" + key] = np.loadtxt(os.path.join(base, latt_name))
        out["ahc_" + key] = np.load(os.path.join(base, "ahc_tens.npy"))
        out["ahcvelo_hw0_" + key] = np.load(os.path.join(base, velo_name))[:, :, 0]
        if tag == "0.900":
            with open(os.path.join(base, "w90files", "FeMn_hr.dat"), "rb") as fh:
                out["hr_dat_" + key] = np.frombuffer(fh.read(), np.uint8)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "femn.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the reference checkout>")
    main(sys.argv[1])
