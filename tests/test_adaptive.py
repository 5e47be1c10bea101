"""Adaptive refinement with the learned proposal (mepinterp_gb300/adaptive.py).

CPU: the sub-mesh indexing (every fine Monkhorst-Pack point belongs to exactly
one coarse cell, centred on it), the cell features and the near-crossing
model.  GPU: refining every cell reproduces the uniform fine mesh; on a small
near-crossing model the learned proposal's AHC error against uniform
refinement by the plain FP64 method is below the coarse mesh's, below a
random choice of the same number of cells, on average below choosing by the
coarse |Omega| alone, and on average (AHC and MEP) below uniform meshes of the
same k-count.
"""
import numpy as np
import pytest

from mepinterp_gb300 import adaptive as AD
from mepinterp_gb300.generator import AU_TO_EV, bloch_hamiltonian, near_crossing_model
from oracle import ref_numpy as O


def test_sub_indices_partition_the_fine_mesh():
    n, s = 5, 3
    cells = np.arange(n ** 3)
    idx = AD.sub_indices(cells, n, s)
    assert idx.shape == (n ** 3, s ** 3)
    assert np.array_equal(np.sort(idx.ravel()), np.arange((n * s) ** 3))
    kc = O.rel_kpts((n, n, n), cells)
    kf = O.rel_kpts((n * s,) * 3, idx.ravel()).reshape(n ** 3, s ** 3, 3)
    off = kf - kc[:, None, :]
    assert np.abs(off).max() < 0.5 / n                               # inside the cell
    assert np.allclose(off.mean(axis=1), 0.0, atol=1e-14)            # centred on it


def test_cell_features_shape_and_neighbours():
    n = 6
    rng = np.random.default_rng(0)
    perk = np.abs(rng.normal(size=(n ** 3, 4)))
    F = AD.cell_features(perk, n)
    assert F.shape == (n ** 3, AD.N_FEATURES) and F.dtype == np.float32
    # column 4 + 13 is the cell itself (offset 0,0,0); column 4 + 14 its +x neighbour
    om = np.sqrt((perk[:, :3] ** 2).sum(1))
    lo = np.log10(om / np.median(om) + 1e-3)
    assert np.allclose(F[:, 4 + 13], lo, atol=1e-6)
    c = 2 + n * 3 + n * n * 4
    assert np.isclose(F[c, 4 + 14], lo[c + 1], atol=1e-6)


def test_near_crossing_model_gaps():
    model, info = near_crossing_model(gaps_ev=(0.002, 0.004))
    nv = model.n_wf // 2
    for k0, g in zip(info["k"], (0.002, 0.004)):
        E = np.linalg.eigvalsh(bloch_hamiltonian(model, k0)[0]) * AU_TO_EV
        assert abs(E[nv] - E[nv - 1] - g) < 1e-6
        assert E[nv - 1] < 0.0 < E[nv]                      # centred on E_F = 0
    for R in range(model.n_R):                              # still Hermitian: H(-R) = H(R)^dag
        j = int(np.argmin(np.abs(model.R_frac + model.R_frac[R]).sum(1)))
        assert np.allclose(model.H[j], model.H[R].conj().T)


def _errs(r, ref):
    return float(np.abs(r["ahc"][:, :, 0] - ref["ahc"][:, :, 0]).max() / np.abs(ref["ahc"][:, :, 0]).max())


def _mep_err(r, ref):
    mep = lambda x: (x["mep_ic"] + x["mep_lc"] + x["mep_cs"]).sum(axis=2)
    return float(np.abs(mep(r) - mep(ref)).max() / np.abs(mep(ref)).max())


@pytest.mark.gpu
def test_refining_every_cell_is_the_uniform_mesh(gpu_lib):
    from mepinterp_gb300 import api
    model, _ = near_crossing_model(gaps_ev=(0.02, 0.04))
    n, s = 6, 2
    job = dict(mp_grid=(n, n, n), ef_lst=np.array([0.0, 0.01]), T_kelvin=0.0, valence_bands=model.n_wf // 2)
    with api.Context(model) as ctx:
        uni = AD.uniform(ctx, job, n, s, precision=api.PREC_FP64)
        full = AD.adaptive(ctx, job, n=n, s=s, frac=1.0, sample_frac=0.0, selector="omega",
                           precision=api.PREC_FP64)
    assert full["cells_refined"] == n ** 3
    for k in AD.SUM_KEYS:
        scale = np.abs(uni[k]).max()
        assert np.abs(full[k] - uni[k]).max() <= 1e-9 * scale, k


@pytest.mark.gpu
def test_learned_proposal_beats_the_method_without_it(gpu_lib):
    """Against uniform refinement by the plain FP64 method on the 64^3 mesh:
    the learned proposal's AHC error is below the coarse mesh's, below random
    cells and on average below |Omega|-ranked cells at the same budget; and, at
    equal cost, its AHC and MEP errors are on average below those of uniform
    meshes with as many k-points (edges m-1, m, m+1 around the cube root of the
    adaptive run's k-count: on a metal a single coarse mesh's error swings with
    its edge, so three of them stand for 'uniform at equal cost')."""
    from mepinterp_gb300 import api
    model, _ = near_crossing_model(gaps_ev=(0.02, 0.03, 0.04, 0.05))
    n, s = 16, 4
    job = dict(mp_grid=(n, n, n), ef_lst=np.array([0.0]), T_kelvin=0.0, valence_bands=model.n_wf // 2)
    with api.Context(model) as ctx:
        uni = AD.uniform(ctx, job, n, s, precision=api.PREC_FP64)
        none = _errs(AD.adaptive(ctx, job, n=n, s=s, selector="none"), uni)
        omega = _errs(AD.adaptive(ctx, job, n=n, s=s, selector="omega"), uni)
        rand = [_errs(AD.adaptive(ctx, job, n=n, s=s, selector="random", seed=sd), uni) for sd in range(3)]
        mlp, mlp_mep, n_eval = [], [], 0
        for sd in range(3):
            r = AD.adaptive(ctx, job, n=n, s=s, selector="mlp", seed=sd)
            assert r["loss_hist"][-1] < 0.1 * r["loss_hist"][0]
            mlp.append(_errs(r, uni))
            mlp_mep.append(_mep_err(r, uni))
            n_eval = r["n_k_evaluated"]
        m_eq = int(round(n_eval ** (1.0 / 3.0)))
        same, same_mep = [], []
        for m in (m_eq - 1, m_eq, m_eq + 1):
            u = ctx.core_worker_loc(dict(job, mp_grid=(m, m, m)), precision=api.PREC_MIXED)
            u = {k: u[k] * (n ** 3 / m ** 3) for k in AD.SUM_KEYS}
            same.append(_errs(u, uni))
            same_mep.append(_mep_err(u, uni))
    assert max(mlp) < 0.7 * none, (mlp, none)
    assert max(mlp) < min(rand), (mlp, rand)
    assert np.mean(mlp) < omega, (mlp, omega)
    assert np.mean(mlp) < np.mean(same), (mlp, same)
    assert np.mean(mlp_mep) < np.mean(same_mep), (mlp_mep, same_mep)


def test_batch_workload_matches_its_recipe():
    """The batched form's 64 models: nWf even in 4..64, R shells 1..3, meshes
    from {32, 48, 64, 96}, 201 Fermi energies over [-1, 1] eV at 290.1 K."""
    from mepinterp_gb300.generator import batch_workload
    work = batch_workload(64)
    assert len(work) == 64
    for m, j in work:
        assert m.n_wf % 2 == 0 and 4 <= m.n_wf <= 64
        assert m.n_R in (27, 125, 343)
        assert j["mp_grid"][0] in (32, 48, 64, 96) and len(set(j["mp_grid"])) == 1
        assert len(j["ef_lst"]) == 201 and abs(j["ef_lst"][-1] * AU_TO_EV - 1.0) < 1e-12
        assert j["T_kelvin"] == 290.1 and j["valence_bands"] == m.n_wf // 2
    again = batch_workload(64)
    assert all(np.array_equal(a[0].H, b[0].H) for a, b in zip(work[:3], again[:3]))   # seeded
