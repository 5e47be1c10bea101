"""Two-rank (gloo, CPU) test of the rank share + k-sum reduction.

Each rank computes its round-robin share of the k-loop -- with the oracle, as
this machine has no GPU -- and the reduced sums must equal a single-rank run,
after which the Fermi selection and normalisation give identical tensors.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from mepinterp_gb300 import output, ranks
from mepinterp_gb300.generator import random_tb_model
from oracle import ref_numpy as O


def _job():
    return dict(mp_grid=(4, 4, 4), ef_lst=np.array([-0.02, 0.0, 0.02]), T_kelvin=0.0, valence_bands=4)


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    model = random_tb_model(n_wf=8, r_max=1, seed=4).as_dict()
    job = _job()

    def compute(k_begin, k_stride):
        return O.run(model, job, k_indices=np.arange(k_begin, 64, k_stride))

    glob = ranks.run_ranked(compute, rank, world)
    if rank == 0:
        np.savez(out_path, **{k: glob[k] for k in ranks.LOC_KEYS}, n_k=glob["n_k"])
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_ranks_gloo(tmp_path):
    out = str(tmp_path / "glob.npz")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    glob = np.load(out)
    model = random_tb_model(n_wf=8, r_max=1, seed=4).as_dict()
    job = _job()
    single = O.run(model, job)
    assert int(glob["n_k"]) == single["n_k"] == 64
    for k in ranks.LOC_KEYS:
        ref = np.asarray(single[k])
        assert np.abs(glob[k] - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1e-300), k
    a = output.integrate_over_k_space({**{k: glob[k] for k in ranks.LOC_KEYS}, "n_k": int(glob["n_k"])},
                                      job["mp_grid"], model["a_latt"], 4)
    b = O.integrate(single, job["mp_grid"], model["a_latt"], 4)
    assert a["eF_idx"] == b["eF_idx"]
    for k in ("ahc_tens", "mep_tens", "kubo_mep_tens"):
        assert np.allclose(a[k], b[k], rtol=1e-12, atol=0)


def test_rank_share_matches_mpi_ki_selector():
    # rank r of P owns 1-based ki with (ki - 1) mod P == r
    for world in (1, 2, 3, 5):
        owned = []
        for r in range(world):
            b, s = ranks.rank_share(r, world)
            owned.append(set(range(b, 30, s)))
        assert set().union(*owned) == set(range(30))
        assert sum(len(o) for o in owned) == 30
    with pytest.raises(ValueError):
        ranks.rank_share(2, 2)
