"""GPU parity of explicit k lists (mepi_job.k_list) and of the per-k output
(mepi_acc.perk) against the oracle.

A k list is sorted into column order for the separable Fourier sums and its
per-k results are scattered back to the caller's order; the tests use
unsorted lists with a repeated index.  Tolerances: the FP64 form's sums 1e-8
and per-k AHC terms 1e-8 relative to the largest entry; the mixed form's sums
1e-6 and its per-k terms 1e-4 (single k-point values computed from FP32
velocities, not k-sums); gaps come from FP64 energies in both forms (1e-9 Ha).
"""
import numpy as np
import pytest

from mepinterp_gb300 import api
from mepinterp_gb300.generator import random_tb_model
from oracle import ref_numpy as O

pytestmark = pytest.mark.gpu

KEYS = ["Ne_sum", "ahc", "mep_ic", "mep_lc", "mep_cs", "kubo_mep_ic", "kubo_mep_lc", "kubo_mep_cs"]
SUM_TOL = {api.PREC_FP64: 1e-8, api.PREC_MIXED: 1e-6}
PERK_TOL = {api.PREC_FP64: 1e-8, api.PREC_MIXED: 1e-4}
GAP_TOL = 1e-9


def _rel(a, b):
    scale = np.abs(b).max()
    return float(np.abs(np.asarray(a) - b).max() / scale) if scale > 0 else float(np.abs(a).max())


def _check(got, ref, prec):
    for k in KEYS:
        assert _rel(got[k], ref[k]) < SUM_TOL[prec], (k, _rel(got[k], ref[k]))
    for c in range(3):
        r = _rel(got["perk"][:, c], ref["perk"][:, c])
        assert r < PERK_TOL[prec], (c, r)
    assert np.abs(got["perk"][:, 3] - ref["perk"][:, 3]).max() < GAP_TOL


@pytest.fixture(scope="module")
def model():
    return random_tb_model(n_wf=10, r_max=2, decay=1.2, seed=31)


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_k_list_with_per_k_output(gpu_lib, model, precision):
    job = dict(mp_grid=(8, 6, 5), ef_lst=np.array([0.01, -0.02]), T_kelvin=0.0, valence_bands=5)
    rng = np.random.default_rng(4)
    klist = rng.permutation(240)[:97]
    klist = np.concatenate([klist, klist[:3]])          # unsorted, with repeats
    ref = O.run(model.as_dict(), job, k_indices=klist, perk=True)
    with api.Context(model) as ctx:
        got = ctx.core_worker_loc(job, precision=precision, k_list=klist, perk=True)
    assert got["n_k"] == klist.size
    _check(got, ref, precision)


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_per_k_output_strided_share(gpu_lib, model, precision):
    """A rank's strided share walked in column order writes each k-point's
    per-k values at its position in the rank's own order."""
    job = dict(mp_grid=(7, 6, 5), ef_lst=np.array([0.0]), T_kelvin=120.0, valence_bands=5)
    kidx = 3 + 4 * np.arange(52)
    ref = O.run(model.as_dict(), job, k_indices=kidx, perk=True)
    with api.Context(model) as ctx:
        got = ctx.core_worker_loc(job, precision=precision, k_begin=3, k_stride=4, perk=True)
    assert got["perk"].shape == (52, 4)
    _check(got, ref, precision)


def test_k_list_rejects_out_of_range(gpu_lib, model):
    job = dict(mp_grid=(4, 4, 4), ef_lst=np.array([0.0]), T_kelvin=0.0, valence_bands=5)
    with api.Context(model) as ctx:
        with pytest.raises(api.MepiError) as e:
            ctx.core_worker_loc(job, k_list=np.array([0, 64]))
        assert e.value.status == 1   # MEPI_ERR_ARG
