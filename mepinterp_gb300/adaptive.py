"""Adaptive k-mesh refinement with a learned proposal.

The reference integrates over a uniform Monkhorst-Pack mesh
(src/k_space.f90:252-256, src/core.f90:165-178).  Near band (anti)crossings
the Berry curvature is sharply peaked and a uniform mesh converges slowly;
this module spends the k-points where they matter instead:

1. a coarse n^3 mesh is run through the CUDA library with the per-k output
   (each k-point's AHC term and the gap across E_F, mepi_acc.perk);
2. every coarse cell gets a feature vector (see :func:`cell_features`): its k,
   log gap, and the log |Omega| of itself and its 26 neighbours;
3. a sample of cells is refined with the s^3 sub-mesh (the fine mesh
   (s n)^3 restricted to the cell, run through mepi_job.k_list): half drawn
   uniformly from all cells, half from the 5% with the smallest coarse gaps
   or the largest coarse |Omega| (the cells that can matter are rare, and a
   uniform sample alone holds too few of them to learn from); the label of a
   cell is how much refinement moves its AHC term,
   log10(eps + sum_c |mean_sub Omega_c - Omega_c(centre)|);
4. the proposal network (include/mepi_mlp.h, trained on the GPU) is trained
   on (features, label) of the sampled cells and predicts the label of every
   cell; the top fraction of the others is refined as well;
5. the sums are re-assembled in the coarse mesh's normalisation:
   acc = coarse - coarse(refined cells) + fine(refined cells) / s^3.

Uniform refinement by the plain FP64 method on the full (s n)^3 mesh stays the
fallback, and the result's error is measured against it (:func:`uniform`).
"""
from __future__ import annotations

import numpy as np

from . import api
from .mlp import Net

SUM_KEYS = ("Ne_sum", "ahc", "mep_ic", "mep_lc", "mep_cs", "kubo_mep_ic", "kubo_mep_lc", "kubo_mep_cs")
N_FEATURES = 31


def sub_indices(cells: np.ndarray, n: int, s: int) -> np.ndarray:
    """Fine-mesh (s n)^3 linear indices (kx fastest) of the s^3 points inside
    each coarse cell.  The Monkhorst-Pack point I = s i + j of the fine mesh
    lies at k_i + (2j + 1 - s) / (2 s n): the sub-mesh of cell i, centred on it."""
    cells = np.asarray(cells, np.int64)
    nf = n * s
    qx, qy, qz = cells % n, (cells // n) % n, cells // (n * n)
    j = np.arange(s)
    fx = (s * qx)[:, None] + j
    fy = (s * qy)[:, None] + j
    fz = (s * qz)[:, None] + j
    idx = fx[:, None, None, :] + nf * fy[:, None, :, None] + nf * nf * fz[:, :, None, None]
    return idx.reshape(cells.size, s ** 3)


def _omega_norm(perk: np.ndarray) -> np.ndarray:
    return np.sqrt((perk[:, :3] ** 2).sum(axis=1))


def cell_features(perk: np.ndarray, n: int) -> np.ndarray:
    """(n^3, 31) features per coarse cell: k (3), log10 gap in eV (1), and
    log10(|Omega| / median |Omega| + 1e-3) of the cell and its 26 periodic
    neighbours (27).  Written column by column into one FP32 array (the
    neighbour columns rolled from the FP32 copy of the cell column)."""
    k = np.arange(n ** 3)
    out = np.empty((n ** 3, N_FEATURES), np.float32)
    q = (k % n, (k // n) % n, k // (n * n))
    for a in range(3):
        out[:, a] = (2.0 * (q[a] + 1) - n - 1) / (2.0 * n)
    out[:, 3] = np.log10(np.maximum(np.abs(perk[:, 3]) * 27.211385, 1e-6))
    om = _omega_norm(perk)
    med = float(np.median(om)) or 1.0
    lo = np.log10(om / med + 1e-3).astype(np.float32).reshape(n, n, n)      # [qz, qy, qx]
    c = 4
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                out[:, c] = np.roll(lo, (-dz, -dy, -dx), axis=(0, 1, 2)).ravel()
                c += 1
    return out


def _job(job: dict, n: int) -> dict:
    j = dict(job)
    j["mp_grid"] = (n, n, n)
    return j


def refine_cells(ctx: api.Context, job: dict, n: int, s: int, cells: np.ndarray, precision: int) -> tuple:
    """(coarse sums over the cells' centres, fine sums over their sub-meshes
    with the per-k output) for a set of coarse cells."""
    cells = np.asarray(cells, np.int64)
    c = ctx.core_worker_loc(_job(job, n), precision=precision, k_list=cells)
    f = ctx.core_worker_loc(_job(job, n * s), precision=precision, k_list=sub_indices(cells, n, s).ravel(),
                            perk=True)
    return c, f


def cell_labels(perk_fine: np.ndarray, perk_coarse_cells: np.ndarray, s: int) -> np.ndarray:
    """log10(1e-3 + sum_c |mean_sub Omega_c - Omega_c(centre)| / scale) per cell
    (scale: median |Omega| of the coarse mesh, folded in by the caller)."""
    m = perk_fine[:, :3].reshape(-1, s ** 3, 3).mean(axis=1)
    return np.abs(m - perk_coarse_cells[:, :3]).sum(axis=1)


def assemble(coarse: dict, parts) -> dict:
    """coarse - coarse(refined) + fine(refined) / s^3 for every (c, f, s) part."""
    out = {k: np.array(coarse[k], copy=True) for k in SUM_KEYS}
    for c, f, s in parts:
        for k in SUM_KEYS:
            out[k] = out[k] - c[k] + f[k] / float(s ** 3)
    return out


def adaptive(ctx: api.Context, job: dict, n: int = 48, s: int = 6, frac: float = 0.02,
             sample_frac: float = 0.01, precision: int = api.PREC_MIXED, seed: int = 0, depth: int = 4,
             epochs: int = 200, batch: int = 256, lr: float = 1e-3, selector: str = "mlp",
             coarse: dict | None = None) -> dict:
    """Adaptive refinement of a job on the n^3 coarse mesh with s^3 sub-meshes.

    ``selector``: "mlp" (the learned proposal, default), "omega" (the coarse
    |Omega| alone), "random" (the same number of cells at random), or "none"
    (the coarse mesh alone).  ``coarse``: the coarse pass's result with its
    per-k output, when the caller has already run it (e.g. inside a batched
    launch); else it is run here.  Returns the sums in the coarse mesh's
    normalisation (so ``output.integrate_over_k_space(res, (n, n, n), ...)``
    normalises them), with bookkeeping: k-points evaluated, cells refined,
    and the network's loss history.
    """
    rng = np.random.default_rng(seed)
    if coarse is None:
        coarse = ctx.core_worker_loc(_job(job, n), precision=precision, perk=True)
    elif "perk" not in coarse or len(coarse["perk"]) != n ** 3:
        raise ValueError("the coarse result needs the per-k output of the whole n^3 mesh")
    perk = coarse["perk"]
    n_cells = n ** 3
    n_sel = int(round(frac * n_cells))
    n_smp = int(round(sample_frac * n_cells))
    info = {"n_coarse": n_cells, "selector": selector}
    if selector == "none":
        res = {k: coarse[k] for k in SUM_KEYS}
        res.update(info, n_k_evaluated=n_cells, cells_refined=0)
        return res
    om = _omega_norm(perk)
    if selector == "omega":
        cells = np.argsort(-om, kind="stable")[:n_sel + n_smp]
        parts = [refine_cells(ctx, job, n, s, cells, precision) + (s,)]
    elif selector == "random":
        cells = rng.choice(n_cells, n_sel + n_smp, replace=False)
        parts = [refine_cells(ctx, job, n, s, cells, precision) + (s,)]
    elif selector == "mlp":
        feats = cell_features(perk, n)
        n_pool = max(int(0.05 * n_cells), n_smp)
        pool = np.union1d(np.argsort(np.abs(perk[:, 3]), kind="stable")[:n_pool // 2],
                          np.argsort(-om, kind="stable")[:n_pool // 2])
        hot = rng.choice(pool, min(n_smp // 2, pool.size), replace=False)
        rest = np.setdiff1d(np.arange(n_cells), hot)
        sample = np.concatenate([hot, rng.choice(rest, n_smp - hot.size, replace=False)])
        c_s, f_s = refine_cells(ctx, job, n, s, sample, precision)
        scale = float(np.median(om)) or 1.0
        lab = np.log10(cell_labels(f_s["perk"], perk[sample], s) / scale + 1e-3).astype(np.float32)
        mu, sd = feats.mean(axis=0), feats.std(axis=0) + 1e-6
        x = feats
        x -= mu                       # in place: the same FP32 operations as (feats - mu) / sd
        x /= sd
        lm, ls = float(lab.mean()), float(lab.std() + 1e-6)
        with Net(N_FEATURES, depth, seed=seed) as net:
            hist = net.train(x[sample], (lab - lm) / ls, epochs=epochs, batch=batch, lr=lr, seed=seed)
            pred = net.forward(x) * ls + lm
        pred[sample] = -np.inf                      # already refined
        cells = np.argsort(-pred, kind="stable")[:n_sel]
        c_t, f_t = refine_cells(ctx, job, n, s, cells, precision)
        parts = [(c_s, f_s, s), (c_t, f_t, s)]
        cells = np.concatenate([sample, cells])
        info["loss_hist"] = hist
        info["label_sample"] = lab
    else:
        raise ValueError(f"unknown selector {selector!r}")
    res = assemble(coarse, parts)
    res.update(info, n_k_evaluated=int(n_cells + cells.size * (s ** 3 + 1)), cells_refined=int(cells.size),
               cells=cells)
    return res


def uniform(ctx: api.Context, job: dict, n: int, s: int, precision: int = api.PREC_FP64) -> dict:
    """Uniform refinement: the (s n)^3 mesh by the given form (plain FP64 by
    default), scaled to the n^3 normalisation of :func:`adaptive`."""
    f = ctx.core_worker_loc(_job(job, n * s), precision=precision)
    return {k: f[k] / float(s ** 3) for k in SUM_KEYS}
