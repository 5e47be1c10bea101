"""Batched form (mepi_run_batch) and autotuner (mepi_autotune).

The batch runs models of uneven band and R counts, each with its own mesh,
Fermi sweep and precision, as one CUDA graph launch; the results must equal
those of separate mepi_run calls bit for bit (same kernels, same order per
model), and the FP64 members match the oracle."""
import numpy as np
import pytest

from mepinterp_gb300 import api
from mepinterp_gb300.generator import random_tb_model
from oracle import ref_numpy as O

pytestmark = pytest.mark.gpu

KEYS = ["Ne_sum", "ahc", "mep_ic", "mep_lc", "mep_cs", "kubo_mep_ic", "kubo_mep_lc", "kubo_mep_cs",
        "velo_ahc", "kubo_ohc"]
SPECS = [  # n_wf, r_max, mesh, precision
    (4, 1, (6, 6, 6), api.PREC_FP64),
    (12, 2, (5, 4, 6), api.PREC_MIXED),
    (20, 1, (4, 4, 4), api.PREC_FP64),
    (32, 2, (4, 4, 3), api.PREC_MIXED),
]


def _job(spec, n_wf):
    return dict(mp_grid=spec[2], ef_lst=np.linspace(-0.02, 0.02, 11), T_kelvin=290.1, valence_bands=n_wf // 2,
                hw_lst=np.array([0.0, 0.01]), eta_smr=0.001)


def test_run_batch_matches_separate_runs(gpu_lib):
    models = [random_tb_model(n_wf=s[0], r_max=s[1], seed=30 + i) for i, s in enumerate(SPECS)]
    jobs = [_job(s, m.n_wf) for s, m in zip(SPECS, models)]
    precs = [s[3] for s in SPECS]
    separate = []
    for m, j, p in zip(models, jobs, precs):
        with api.Context(m) as c:
            separate.append(c.core_worker_loc(j, precision=p))
    ctxs = [api.Context(m) for m in models]
    try:
        batch, ms = api.run_batch(ctxs, jobs, precs)
    finally:
        for c in ctxs:
            c.close()
    assert ms > 0.0
    for a, b in zip(batch, separate):
        assert a["n_k"] == b["n_k"]
        for k in KEYS:
            assert np.array_equal(a[k], b[k]), k
    for i in (0, 2):   # FP64 members against the oracle
        ref = O.run(models[i].as_dict(), jobs[i])
        for k in KEYS:
            scale = np.abs(ref[k]).max()
            assert np.abs(batch[i][k] - ref[k]).max() <= 1e-8 * scale, k


def test_run_batch_rejects_repeated_context(gpu_lib):
    m = random_tb_model(n_wf=8, r_max=1, seed=1)
    job = dict(mp_grid=(3, 3, 3), ef_lst=[0.0], valence_bands=4)
    with api.Context(m) as c:
        with pytest.raises(api.MepiError) as e:
            api.run_batch([c, c], [job, job], api.PREC_FP64)
        assert e.value.status == api.ERR_ARG


def test_autotune(gpu_lib):
    m = random_tb_model(n_wf=16, r_max=2, seed=9)
    job = dict(mp_grid=(16, 16, 16), ef_lst=[0.0], T_kelvin=0.0, valence_bands=8)
    with api.Context(m) as c:
        base = c.core_worker_loc(job, precision=api.PREC_MIXED)
        t = c.autotune(job, precision=api.PREC_MIXED, sample_k=2048)
        assert t["jacobi_threads"] in (64, 128, 256) and t["jacobi_kblock"] in (4, 8, 16)
        assert t["chunk_k"] in (16384, 65536) and t["k_per_s"] > 0
        assert c.get_tuning() == t
        tuned = c.core_worker_loc(job, precision=api.PREC_MIXED)
    for k in ("ahc", "mep_ic", "kubo_mep_ic"):
        assert np.abs(tuned[k] - base[k]).max() <= 1e-6 * np.abs(base[k]).max(), k
    # a later context of the same kind starts from the recorded shapes
    with api.Context(m) as c2:
        assert c2.get_tuning() == t
