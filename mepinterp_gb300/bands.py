"""Band-structure mode: ``band_worker`` of src/band_calc.f90:30-92.

Interpolates the energies (and, with ``do_write_velo``, the velocities) at the
k-points of a ``kpts`` file through the CUDA library (``mepi_interp_k``) and
writes them in the reference's formats:

* ``kpts``: kptsgen.pl output read by read_kptsgen_pl_file
  (src/file_io.f90:451-476): a first line ``num_kpts <x>``, then one line
  ``kx ky kz weight`` per k-point in lattice units;
* ``raw/enK.<7-digit k index>``: the band energies of one k-point as raw FP64
  (write_en_binary, src/file_io.f90:57-70; k index 1-based);
* ``out/eBands.dat``: every (k, band) with the relative k-point and the energy
  in Hartree (write_en_global, src/file_io.f90:116-143);
* ``out//velo/velo_Vka.<7-digit k index>``: V^x_nm per k-point
  (write_velo, src/file_io.f90:146-182).
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import api


def read_kpts_file(path: str) -> np.ndarray:
    """k-points (num_kpts, 3) of a kptsgen.pl file."""
    with open(path) as fh:
        first = fh.readline().split()
        n = int(first[0])
        rows = []
        for _ in range(n):
            parts = fh.readline().split()
            rows.append([float(x) for x in parts[:3]])
    return np.asarray(rows, dtype=np.float64).reshape(n, 3)


def write_kpts_file(path: str, kpts: np.ndarray) -> None:
    """A kptsgen.pl-style file (weights 1) for the given k-points."""
    kpts = np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
    with open(path, "w") as fh:
        fh.write(f"{kpts.shape[0]} 1.0\n")
        for k in kpts:
            fh.write(f"{k[0]:.10f} {k[1]:.10f} {k[2]:.10f} 1.0\n")


def k_path(corners, n_per_segment: int) -> np.ndarray:
    """Straight segments between high-symmetry points (lattice units), as a
    kpts file lists them: n_per_segment points per segment, end point included
    once."""
    corners = np.asarray(corners, dtype=np.float64)
    pts = []
    for a, b in zip(corners[:-1], corners[1:]):
        for t in np.arange(n_per_segment) / n_per_segment:
            pts.append(a + t * (b - a))
    pts.append(corners[-1])
    return np.asarray(pts)


def write_en_binary(raw_dir: str, ki: int, e_bands: np.ndarray) -> str:
    path = os.path.join(raw_dir, f"enK.{ki:07d}")
    np.asarray(e_bands, dtype="<f8").tofile(path)
    return path


def read_en_binary(raw_dir: str, ki: int) -> np.ndarray:
    return np.fromfile(os.path.join(raw_dir, f"enK.{ki:07d}"), dtype="<f8")


def write_en_global(out_dir: str, kpts: np.ndarray, energies: np.ndarray) -> str:
    path = os.path.join(out_dir, "eBands.dat")
    with open(path, "w") as fh:
        fh.write(" # energies interpolated by MEPinterp program, written " + time.ctime() + "\n")
        fh.write(" # first 3 columns give the relative k-mesh, 4th column are the enegies\n")
        fh.write(" # Kpt_idx  K_x (frac)       K_y (frac)        K_z (frac)       Energy (Hartree)  \n")
        for qi, (k, e) in enumerate(zip(kpts, energies), start=1):
            head = f"{qi:7d}\t" + "".join(f"{x:16.8f}" for x in k)
            for band in e:
                fh.write(f"{head}\t{band:18.8f}\n")
    return path


def read_en_global(path: str):
    """(k index, k (3), energy) columns of an eBands.dat file."""
    data = np.loadtxt(path, comments="#")
    return data[:, 0].astype(int), data[:, 1:4], data[:, 4]


def write_velo(velo_dir: str, ki: int, V: np.ndarray) -> str:
    """V (3, N, N) complex of one k-point."""
    path = os.path.join(velo_dir, f"velo_Vka.{ki:07d}")
    with open(path, "w") as fh:
        fh.write(" #interpolated velocities\n")
        fh.write(" # x |\t n\t\t|\tm \t|\treal(V^x_nm)  |\t\timag(Vx_nm)\n")
        fh.write(" #-----------------------------------------------------------------------\n")
        for x in range(3):
            for m in range(V.shape[2]):
                for n in range(V.shape[1]):
                    v = V[x, n, m]
                    fh.write(f"\t{x + 1:1d}\t\t{n + 1:3d}\t\t{m + 1:3d}\t\t{v.real:16.8f}\t{v.imag:16.8f}\n")
            fh.write(" #----------------------------------------------------------------------\n")
    return path


def band_worker(workdir: str, model, do_write_velo: bool = False, precision: int = api.PREC_FP64,
                rank: int = 0, nprocs: int = 1) -> dict:
    """The k-points of ``workdir/kpts`` owned by this rank (ki = rank+1,
    rank+1+nprocs, ..., 1-based, as the reference's loop); rank 0 also writes
    eBands.dat from all raw files."""
    kpath = os.path.join(workdir, "kpts")
    if not os.path.exists(kpath):
        raise FileNotFoundError("for bandstructure calculations a kpts file has to be provided")
    kpts = read_kpts_file(kpath)
    raw_dir = os.path.join(workdir, "raw")
    out_dir = os.path.join(workdir, "out")
    velo_dir = os.path.join(out_dir, "", "velo")
    os.makedirs(raw_dir, exist_ok=True)
    os.makedirs(out_dir, exist_ok=True)
    if do_write_velo:
        os.makedirs(velo_dir, exist_ok=True)
    mine = np.arange(rank, kpts.shape[0], nprocs)
    with api.Context(model) as ctx:
        E, V, _, _ = ctx.get_wann_interp(kpts[mine], precision=precision)
    for j, ki0 in enumerate(mine):
        write_en_binary(raw_dir, int(ki0) + 1, E[j])
        if do_write_velo:
            write_velo(velo_dir, int(ki0) + 1, V[j])
    written = None
    if rank == 0 and nprocs == 1:
        allE = np.stack([read_en_binary(raw_dir, ki + 1) for ki in range(kpts.shape[0])])
        written = write_en_global(out_dir, kpts, allE)
    return {"kpts": kpts, "energies": E, "eBands": written, "n_k": int(mine.size)}
