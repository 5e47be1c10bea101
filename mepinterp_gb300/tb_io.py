"""Tight-binding input in the reference's file formats.

Readers
  read_hr_file   Wannier90 ``<seed>_hr.dat`` (src/file_io.f90:663-746): header
                 line, n_wf, nrpts, the Wigner-Seitz degeneracies (15 per line,
                 read and ignored as in the reference, D8), then nrpts * n_wf^2
                 lines ``R1 R2 R3 m n Re Im`` (eV); |Re|, |Im| < 1e-7 are set to
                 zero (:732-733) and H is converted to Hartree (:741).
  read_r_file    ``<seed>_r.dat`` (src/file_io.f90:750-795): header, n_wf, then
                 lines ``R1 R2 R3 m n Re_x Im_x Re_y Im_y Re_z Im_z`` (Angstrom)
                 in the same R order as _hr.dat, converted to bohr (:790).  The
                 reference passes a doubled suffix to this reader
                 (src/file_io.f90:838, D6); the file opened here is
                 ``<seed>_r.dat``.
  read_tb_basis  both of the above, like src/file_io.f90:800-860 (the _tb.dat
                 route, whose R vectors are stored Cartesian but used as
                 fractional (D7), is not offered).
  read_input_cfg the INI-style ``input.cfg`` of src/input_paras.f90:99-160.

Writers (the formats of scripts/tb_input_writer.py:42-190): write_hr_file,
write_r_file, write_input_cfg.
"""
from __future__ import annotations

import configparser
import datetime
import os
import warnings
from typing import Optional

import numpy as np

from .generator import AU_TO_ANGSTROM, AU_TO_EV, TBModel


class TBFormatError(ValueError):
    pass


def _lines(path):
    with open(path) as fh:
        return [ln for ln in fh.read().split("\n")]


def read_hr_file(path: str):
    """Return (R_frac (nR,3), H (nR,N,N) complex Hartree, degeneracies (nR,))."""
    lines = _lines(path)
    try:
        n_wf = int(lines[1].split()[0])
        n_r = int(lines[2].split()[0])
    except (IndexError, ValueError) as exc:
        raise TBFormatError(f"{path}: bad header") from exc
    deg = []
    i = 3
    while len(deg) < n_r:
        if i >= len(lines):
            raise TBFormatError(f"{path}: issue reading Wigner Seitz degeneracy")
        deg.extend(int(x) for x in lines[i].split())
        i += 1
    if len(deg) != n_r:
        raise TBFormatError(f"{path}: issue reading Wigner Seitz degeneracy (idx/=f_nSC)")
    body = [ln.split() for ln in lines[i:] if ln.strip()]
    if len(body) < n_r * n_wf * n_wf:
        raise TBFormatError(f"{path}: expected {n_r * n_wf * n_wf} matrix lines, found {len(body)}")
    arr = np.array([[float(x) for x in row[:7]] for row in body[: n_r * n_wf * n_wf]])
    arr = arr.reshape(n_r, n_wf * n_wf, 7)
    R = arr[:, 0, :3].copy()
    # an R vector that changes inside its block: the reference warns, keeps the
    # block's first R and still stores the element (src/file_io.f90:720-727)
    bad = np.argwhere(np.any(np.abs(arr[:, :, :3] - R[:, None, :]) >= 1e-14, axis=2))
    for sc, wf in bad:
        warnings.warn(f"[read_hr_file]: WARNING unexpected new R_vect={arr[sc, wf, :3].tolist()} "
                      f"m={int(arr[sc, wf, 3])} n={int(arr[sc, wf, 4])} wf={wf + 1} sc={sc + 1} "
                      f"expected R_vect={R[sc].tolist()}", RuntimeWarning, stacklevel=2)
    m = arr[:, :, 3].astype(int) - 1
    n = arr[:, :, 4].astype(int) - 1
    re = arr[:, :, 5].copy()
    im = arr[:, :, 6].copy()
    re[np.abs(re) < 1e-7] = 0.0
    im[np.abs(im) < 1e-7] = 0.0
    H = np.zeros((n_r, n_wf, n_wf), np.complex128)
    for r in range(n_r):
        H[r, m[r], n[r]] = re[r] + 1j * im[r]
    return R, H / AU_TO_EV, np.asarray(deg)


def read_r_file(path: str, R_frac: np.ndarray):
    """Return r (nR,3,N,N) complex in bohr; R order must match _hr.dat."""
    lines = _lines(path)
    n_wf = int(lines[1].split()[0])
    n_r = R_frac.shape[0]
    body = [ln.split() for ln in lines[2:] if ln.strip()]
    if len(body) < n_r * n_wf * n_wf:
        raise TBFormatError(f"{path}: expected {n_r * n_wf * n_wf} lines, found {len(body)}")
    arr = np.array([[float(x) for x in row[:11]] for row in body[: n_r * n_wf * n_wf]])
    arr = arr.reshape(n_r, n_wf * n_wf, 11)
    if not np.all(np.abs(arr[:, :, :3] - R_frac[:, None, :]) < 1e-14):
        raise TBFormatError(f"{path}: different R_vect order in _hr.dat and _r.dat file")
    m = arr[:, :, 3].astype(int) - 1
    n = arr[:, :, 4].astype(int) - 1
    r = np.zeros((n_r, 3, n_wf, n_wf), np.complex128)
    for R in range(n_r):
        for a in range(3):
            r[R, a, m[R], n[R]] = arr[R, :, 5 + 2 * a] + 1j * arr[R, :, 6 + 2 * a]
    return r / AU_TO_ANGSTROM


def read_tb_basis(w90_dir: str, seed: str, wf_centers: Optional[np.ndarray] = None,
                  a_latt: Optional[np.ndarray] = None) -> TBModel:
    """src/file_io.f90:800-860: mandatory _hr.dat, optional _r.dat."""
    hr = os.path.join(w90_dir, seed + "_hr.dat")
    if not os.path.exists(hr):
        raise FileNotFoundError(f'"{hr}" does not exist')
    R, H, _ = read_hr_file(hr)
    rpath = os.path.join(w90_dir, seed + "_r.dat")
    r = read_r_file(rpath, R) if os.path.exists(rpath) else None
    if r is not None and r.shape[2] != H.shape[1]:
        raise TBFormatError("r_mat and H_mat have different basis")
    return TBModel(R_frac=R, H=H, r=r, wf_centers=wf_centers,
                   a_latt=np.eye(3) if a_latt is None else np.asarray(a_latt, np.float64))


def write_hr_file(path: str, model: TBModel, header: str = "tight-binding model") -> None:
    """Wannier90 _hr.dat (eV), the layout of scripts/tb_input_writer.py:42-72."""
    H = np.asarray(model.H) * AU_TO_EV
    n_r, n_wf, _ = H.shape
    with open(path, "w") as out:
        out.write(f"# {header} written {datetime.date.today().isoformat()}\n")
        out.write(f"{n_wf}\n{n_r}\n")
        for s in range(0, n_r, 15):
            out.write(" ".join("1" for _ in range(min(15, n_r - s))) + "\n")
        for r in range(n_r):
            Rv = model.R_frac[r]
            for nn in range(n_wf):
                for mm in range(n_wf):
                    v = H[r, mm, nn]
                    out.write(f"{int(round(Rv[0]))} {int(round(Rv[1]))} {int(round(Rv[2]))} {mm + 1} {nn + 1} "
                              f"{v.real:.12e} {v.imag:.12e}\n")


def write_r_file(path: str, model: TBModel, header: str = "position operator") -> None:
    """_r.dat (Angstrom), the layout of scripts/tb_input_writer.py:75-92."""
    if model.r is None:
        raise ValueError("model has no position operator")
    r = np.asarray(model.r) * AU_TO_ANGSTROM
    n_r, _, n_wf, _ = r.shape
    with open(path, "w") as out:
        out.write(f"# {header} written {datetime.date.today().isoformat()}\n{n_wf}\n")
        for R in range(n_r):
            Rv = model.R_frac[R]
            for nn in range(n_wf):
                for mm in range(n_wf):
                    vals = " ".join(f"{r[R, a, mm, nn].real:.12e} {r[R, a, mm, nn].imag:.12e}" for a in range(3))
                    out.write(f"{int(round(Rv[0]))} {int(round(Rv[1]))} {int(round(Rv[2]))} {mm + 1} {nn + 1} {vals}\n")


def write_input_cfg(path: str, *, seed_name: str, a_latt: np.ndarray, mp_grid, valence_bands: int,
                    wf_centers: Optional[np.ndarray] = None, eF_min=0.0, eF_max=0.0, N_eF=1, Tkelvin=0.0,
                    eta_smearing=0.1, kubo_tol=1e-5, do_mep=True, do_kubo=True, do_ahc=True,
                    do_gauge_trafo=True, use_cart_velo=False, n_hw=1, hw_min=0.0, hw_max=0.0,
                    plot_bands=False, do_write_velo=False) -> None:
    """input.cfg with the sections of scripts/tb_input_writer.py:102-190."""
    a = np.asarray(a_latt, np.float64)
    T = lambda b: "T" if b else "F"
    lines = ["[jobs]", f"    plot_bands={T(plot_bands)}", "    debug_mode=F", "    R_vect_float=F",
             f"    do_write_velo={T(do_write_velo)}",
             f"    do_mep={T(do_mep)}", f"    do_kubo={T(do_kubo)}", f"    do_ahc={T(do_ahc)}", "    do_opt=F",
             "    do_gyro=F", "", "[unitCell]"]
    for i in range(3):
        lines.append(f"    a{i + 1}= {float(a[i, 0])!r} {float(a[i, 1])!r} {float(a[i, 2])!r}")
    lines += ["    a0= 1.0", "", "[wannBase]", f"    seed_name= {seed_name}"]
    if wf_centers is not None:
        tau = np.asarray(wf_centers)
        lines.append(f"    N_wf= {tau.shape[0]}")
        for c, nm in enumerate("xyz"):
            lines.append(f"    wf_centers_{nm}= " + " ".join(repr(float(x)) for x in tau[:, c]))
    else:
        lines.append("    N_wf= 0")
    lines += ["", "[wannInterp]", f"    use_cart_velo= {T(use_cart_velo)}", f"    doGaugeTrafo= {T(do_gauge_trafo)}",
              f"    mp_grid= {mp_grid[0]} {mp_grid[1]} {mp_grid[2]}", "", "[Fermi]", f"    N_eF= {N_eF}",
              f"    eF_min= {float(eF_min)!r}", f"    eF_max= {float(eF_max)!r}", f"    Tkelvin= {float(Tkelvin)!r}",
              f"    eta_smearing= {float(eta_smearing)!r}", f"    kuboTol= {float(kubo_tol)!r}", "", "[MEP]",
              f"    valence_bands= {valence_bands}", "    do_write_mep_bands= T", "", "[Laser]",
              f"    N_hw= {n_hw}", f"    hw_min= {float(hw_min)!r}", f"    hw_max= {float(hw_max)!r}", ""]
    with open(path, "w") as out:
        out.write("\n".join(lines))


def _linspace(lo: float, hi: float, n: int) -> np.ndarray:
    """get_linspace, src/matrix_math.f90:74-100: n points from lo to hi, or [lo]."""
    if n > 1:
        return np.array([lo + i * (hi - lo) / (n - 1) for i in range(n)])
    return np.array([lo])


def _flag(v: str) -> bool:
    v = v.strip().strip(".").lower()
    return v in ("t", "true", "1", "yes")


def read_input_cfg(path: str) -> dict:
    """Parse input.cfg (src/input_paras.f90:99-181) into a settings dict.

    Energies are converted from eV to Hartree (:171-178) and a_latt is built as
    a0 * (a1; a2; a3) with row i = a_i (:165-168).
    """
    cp = configparser.ConfigParser(inline_comment_prefixes=("#", "!"))
    with open(path) as fh:
        cp.read_string(fh.read())

    def get(sec, key, default=None):
        for s in cp.sections():
            if s.lower() == sec.lower():
                for k, v in cp.items(s):
                    if k.lower() == key.lower():
                        return v
        return default

    vec = lambda s: np.array([float(x) for x in s.replace(",", " ").split()])
    a0 = float(get("unitCell", "a0", "1.0"))
    a_latt = np.vstack([vec(get("unitCell", f"a{i}")) for i in (1, 2, 3)]) * a0
    n_wf = int(get("wannBase", "N_wf", "0"))
    tau = None
    if n_wf > 0:
        tau = np.stack([vec(get("wannBase", f"wf_centers_{c}")) for c in "xyz"], axis=1)[:n_wf]
    n_ef = int(get("Fermi", "N_eF", "1"))
    ef_min = float(get("Fermi", "eF_min", "0")) / AU_TO_EV
    ef_max = float(get("Fermi", "eF_max", "0")) / AU_TO_EV
    ef_lst = _linspace(ef_min, ef_max, n_ef)
    return {
        "seed_name": get("wannBase", "seed_name", "wf1").strip(),
        "a_latt": a_latt, "wf_centers": tau,
        "mp_grid": tuple(int(x) for x in get("wannInterp", "mp_grid").split()),
        "use_cart_velo": _flag(get("wannInterp", "use_cart_velo", "F")),
        "do_gauge_trafo": _flag(get("wannInterp", "doGaugeTrafo", "T")),
        "ef_lst": ef_lst, "T_kelvin": float(get("Fermi", "Tkelvin", "0")),
        "eta": float(get("Fermi", "eta_smearing", "0")) / AU_TO_EV,
        "kubo_tol": float(get("Fermi", "kuboTol", "1e-5")),
        "valence_bands": int(get("MEP", "valence_bands", "0")),
        "do_write_mep_bands": _flag(get("MEP", "do_write_mep_bands", "F")),
        "do_mep": _flag(get("jobs", "do_mep", "F")), "do_kubo": _flag(get("jobs", "do_kubo", "F")),
        "do_ahc": _flag(get("jobs", "do_ahc", "F")),
        "hw_lst": _linspace(float(get("Laser", "hw_min", "0")) / AU_TO_EV, float(get("Laser", "hw_max", "0")) / AU_TO_EV,
                            int(get("Laser", "N_hw", "1"))),
        "plot_bands": _flag(get("jobs", "plot_bands", "F")),
        "do_write_velo": _flag(get("jobs", "do_write_velo", "F")),
    }
