"""Output stage of core_worker: Fermi-level selection, k-space normalisation
and the .npy files.

fermi_selector          src/core.f90:317-415 -- N_el(E_F) = Ne_sum / n_k; the
                        first E_F index minimising |N_el - valence_bands| wins;
                        occ.dat lists E_F (eV) and N_el.
integrate_over_k_space  src/core.f90:419-561 (+ mep_sum_bands :570-603) -- sums
                        the Niu MEP over valence bands, keeps only the selected
                        E_F slice of the Kubo tensors (D10) and divides by
                        |V_cell| N_k (normalize_k_int, src/k_space.f90:81-202).
write_outputs           the file names of src/file_io.f90:186-359 (with
                        ahcVELO.npy / ohcVELO.npy of velo_ahc_tens and
                        kubo_ohc_tens, and hw_lst.npy), written with
                        Fortran ordering as NPY-for-Fortran does; additionally
                        the full Fermi sweeps (*_sweep.npy), which the
                        reference accumulates but does not write.
"""
from __future__ import annotations

import os

import numpy as np

from .generator import AU_TO_EV


def unit_volume(a_latt) -> float:
    a = np.asarray(a_latt, np.float64)
    # set_recip_latt uses the columns of a_latt (src/k_space.f90:274-278)
    return float(np.dot(np.cross(a[:, 0], a[:, 1]), a[:, 2]))


def fermi_selector(n_k_glob: int, Ne_sum, valence_bands: int) -> int:
    Ne = np.asarray(Ne_sum, np.float64) / float(n_k_glob)
    best, err = 0, abs(Ne[0] - float(valence_bands))
    for i in range(1, Ne.size):
        e = abs(Ne[i] - float(valence_bands))
        if e < err:
            best, err = i, e
    return best


def integrate_over_k_space(loc: dict, mp_grid, a_latt, valence_bands: int, n_k_glob=None) -> dict:
    """Normalised tensors from the unnormalised local sums of one (or all) ranks."""
    n_k_glob = int(loc["n_k"] if n_k_glob is None else n_k_glob)
    e = fermi_selector(n_k_glob, loc["Ne_sum"], valence_bands)
    nk = int(mp_grid[0]) * int(mp_grid[1]) * int(mp_grid[2])
    norm = abs(unit_volume(a_latt) * nk) if nk > 0 else 1.0
    out = {"eF_idx": e, "n_k": n_k_glob, "Ne": np.asarray(loc["Ne_sum"]) / n_k_glob}
    for key in ("mep_ic", "mep_lc", "mep_cs"):
        out[key] = np.asarray(loc[key]).sum(axis=-1) / norm
    out["mep_tens"] = out["mep_ic"] + out["mep_lc"] + out["mep_cs"]
    out["mep_bands"] = (np.asarray(loc["mep_ic"]) + np.asarray(loc["mep_lc"]) + np.asarray(loc["mep_cs"])) / norm
    for key in ("kubo_mep_ic", "kubo_mep_lc", "kubo_mep_cs"):
        out[key] = np.asarray(loc[key])[:, :, e] / norm
        out[key + "_sweep"] = np.asarray(loc[key]) / norm
    out["kubo_mep_tens"] = out["kubo_mep_ic"] + out["kubo_mep_lc"] + out["kubo_mep_cs"]
    out["ahc_tens"] = np.asarray(loc["ahc"])[:, :, e] / norm
    out["ahc_sweep"] = np.asarray(loc["ahc"]) / norm
    if "velo_ahc" in loc:                      # src/core.f90:501-508: the selected E_F slice
        out["ahc_velo"] = np.asarray(loc["velo_ahc"])[:, :, :, e] / norm
        out["ohc_velo"] = np.asarray(loc["kubo_ohc"])[:, :, :, e] / norm
    return out


def write_outputs(out_dir: str, res: dict, ef_lst, do_mep=True, do_kubo=True, do_ahc=True,
                  write_mep_bands=True, hw_lst=None) -> list:
    os.makedirs(out_dir, exist_ok=True)
    written = []

    def save(name, arr):
        p = os.path.join(out_dir, name)
        np.save(p, np.asfortranarray(arr))
        written.append(p)

    with open(os.path.join(out_dir, "occ.dat"), "w") as fh:
        for ef, ne in zip(np.asarray(ef_lst), res["Ne"]):
            fh.write(f"{ef * AU_TO_EV:16.8f}\t{ne:16.8f}\n")
    if do_mep:
        for k in ("mep_ic", "mep_lc", "mep_cs", "mep_tens"):
            save(k + ".npy", res[k])
        if write_mep_bands:
            save("mep_bands.npy", res["mep_bands"])
    if do_kubo:
        for k in ("kubo_mep_ic", "kubo_mep_lc", "kubo_mep_cs", "kubo_mep_tens"):
            save(k + ".npy", res[k])
        for k in ("kubo_mep_ic", "kubo_mep_lc", "kubo_mep_cs"):
            save(k + "_sweep.npy", res[k + "_sweep"])
    if hw_lst is not None and len(hw_lst) > 1:   # write_hw_list, src/file_io.f90:186-214 (eV)
        save("hw_lst.npy", np.asarray(hw_lst, np.float64) * AU_TO_EV)
    if do_ahc:
        save("ahc_tens.npy", res["ahc_tens"])
        save("ahc_sweep.npy", res["ahc_sweep"])
        if "ahc_velo" in res:                  # write_ahc_tensor, src/file_io.f90:340-359
            save("ahcVELO.npy", res["ahc_velo"])
            save("ohcVELO.npy", res["ohc_velo"])
    return written
