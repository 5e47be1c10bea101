"""Drop-in driver: ``python -m mepinterp_gb300.cli [workdir]``.

Does what ``mepInterp`` does for the AHC / MEP jobs (src/main.f90:24-45 ->
src/core.f90:79-298) and, with ``jobs%plot_bands = T``, for the band-structure
mode (src/band_calc.f90:30-92, see ``bands.py``) on one GPU: reads ``./input.cfg`` and
``./w90files/<seed>_hr.dat`` (+ ``_r.dat``), runs the k-loop through the CUDA
library (MEPI_PREC_FP64 by default, ``--mixed`` for the mixed form), selects
the Fermi level, normalises and writes ``./out/*.npy``.  ``--rank R --nprocs P``
runs the share of rank R of a P-way round-robin split (mpi_ki_selector,
src/mpi_comm.f90:80-99) and writes the unnormalised local sums to
``out/loc_rank<R>.npz`` for a later ``--reduce P``.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from . import api, bands, output, tb_io


def main(argv=None) -> int:
    p = argparse.ArgumentParser(prog="mepinterp_gb300.cli")
    p.add_argument("workdir", nargs="?", default=".")
    p.add_argument("--mixed", action="store_true", help="mixed precision form")
    p.add_argument("--rank", type=int, default=0)
    p.add_argument("--nprocs", type=int, default=1)
    p.add_argument("--reduce", type=int, default=0, help="combine out/loc_rank*.npz of this many ranks")
    a = p.parse_args(argv)
    cfg = tb_io.read_input_cfg(os.path.join(a.workdir, "input.cfg"))
    out_dir = os.path.join(a.workdir, "out")
    keys = ["Ne_sum", "ahc", "mep_ic", "mep_lc", "mep_cs", "kubo_mep_ic", "kubo_mep_lc", "kubo_mep_cs"]
    if cfg["do_ahc"]:
        keys += ["velo_ahc", "kubo_ohc"]
    if a.reduce:
        parts = [np.load(os.path.join(out_dir, f"loc_rank{r}.npz")) for r in range(a.reduce)]
        loc = {k: sum(np.asarray(pp[k]) for pp in parts) for k in keys}
        loc["n_k"] = int(sum(int(pp["n_k"]) for pp in parts))
    else:
        model = tb_io.read_tb_basis(os.path.join(a.workdir, "w90files"), cfg["seed_name"],
                                    wf_centers=cfg["wf_centers"], a_latt=cfg["a_latt"])
        model.do_gauge_trafo = cfg["do_gauge_trafo"]
        model.use_cart_velo = cfg["use_cart_velo"]
        model.kubo_tol = cfg["kubo_tol"]
        if cfg.get("plot_bands"):
            prec = api.PREC_MIXED if a.mixed else api.PREC_FP64
            r = bands.band_worker(a.workdir, model, do_write_velo=cfg.get("do_write_velo", False), precision=prec,
                                  rank=a.rank, nprocs=a.nprocs)
            print(f"interpolated {r['n_k']} of {r['kpts'].shape[0]} kpts")
            return 0
        job = dict(mp_grid=cfg["mp_grid"], ef_lst=cfg["ef_lst"], T_kelvin=cfg["T_kelvin"],
                   valence_bands=cfg["valence_bands"], do_mep=cfg["do_mep"], do_kubo=cfg["do_kubo"],
                   do_ahc=cfg["do_ahc"], hw_lst=cfg["hw_lst"], eta_smr=cfg["eta"])
        prec = api.PREC_MIXED if a.mixed else api.PREC_FP64
        with api.Context(model) as ctx:
            loc = ctx.core_worker_loc(job, precision=prec, k_begin=a.rank, k_stride=a.nprocs)
        if a.nprocs > 1:
            os.makedirs(out_dir, exist_ok=True)
            np.savez(os.path.join(out_dir, f"loc_rank{a.rank}.npz"), **{k: loc[k] for k in keys}, n_k=loc["n_k"])
            return 0
    res = output.integrate_over_k_space(loc, cfg["mp_grid"], cfg["a_latt"], cfg["valence_bands"])
    files = output.write_outputs(out_dir, res, cfg["ef_lst"], do_mep=cfg["do_mep"], do_kubo=cfg["do_kubo"],
                                 do_ahc=cfg["do_ahc"], write_mep_bands=cfg["do_write_mep_bands"],
                                 hw_lst=cfg["hw_lst"])
    print(f"chosen fermi energy {cfg['ef_lst'][res['eF_idx']] * 27.211385:.6f} eV; wrote {len(files)} files to {out_dir}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
