"""Seeded synthetic tight-binding models for the benchmark workloads.

The reference's own drivers write a tight-binding basis in Wannier90 text
format (scripts/tb_input_writer.py:42-92) and an ``input.cfg``
(scripts/tb_input_writer.py:102-190) before running the Fortran core.  This
module produces the same kind of input from a seed, in atomic units, as the
arrays the C ABI takes; :mod:`mepinterp_gb300.tb_io` writes them out in the
reference's text formats when files are wanted.

Model recipe (all energies in eV before conversion, lengths in Angstrom):

* ``n_orb`` orbitals x 2 spins, ``n_wf = 2 n_orb``; the orbitals sit on a fixed
  4-site pattern inside the cell (repeated with a small shift when n_orb > 4),
  the same centres for both spins;
* R runs over the cube {-r_max..r_max}^3 (nR = (2 r_max + 1)^3);
* H(R) for R != 0 in the upper half-space: complex N(0,1) * exp(-|R| / lam),
  H(-R) = H(R)^dag;  H(0): Hermitian N(0,1) off-diagonal plus onsite U[-2,2];
* spin-orbit-like imaginary hoppings 0.1 eV * i * s_z on the nearest
  neighbours (|R| = 1), kept Hermitian through H(-R) = H(R)^dag;
* r(R) ~ N(0, 0.05) Angstrom per Cartesian component, Hermitian the same way;
* cubic cell of edge ``a_bohr`` (5 bohr by default).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

AU_TO_EV = 27.211385          # src/constants.f90:19
AU_TO_ANGSTROM = 0.52917721092  # src/constants.f90:18

_SITES = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.0, 0.5]])


@dataclass
class TBModel:
    """A tight-binding basis in atomic units (Hartree, bohr), C-order arrays.

    ``H[r, n, m]`` is the reference's ``H_real(n, m, r)``; ``r[R, a, n, m]`` is
    ``r_real(a, n, m, R)``; ``R_frac[r, :]`` is ``R_frac(:, r)``;
    ``wf_centers[n, :]`` is ``wf_centers(:, n)`` (``None`` selects the Wannier
    phase convention); ``a_latt`` is the reference's ``a_latt`` (row i = a_i).
    """
    R_frac: np.ndarray
    H: np.ndarray
    r: Optional[np.ndarray] = None
    wf_centers: Optional[np.ndarray] = None
    a_latt: np.ndarray = field(default_factory=lambda: 5.0 * np.eye(3))
    do_gauge_trafo: bool = True
    use_cart_velo: bool = False
    semantics: str = "ref"
    kubo_tol: float = 1e-5

    @property
    def n_wf(self) -> int:
        return int(self.H.shape[1])

    @property
    def n_R(self) -> int:
        return int(self.H.shape[0])

    def as_dict(self) -> dict:
        return dict(R_frac=self.R_frac, H=self.H, r=self.r, wf_centers=self.wf_centers,
                    a_latt=self.a_latt, do_gauge_trafo=self.do_gauge_trafo,
                    use_cart_velo=self.use_cart_velo, semantics=self.semantics,
                    kubo_tol=self.kubo_tol)


def _cube(r_max: int) -> np.ndarray:
    rng = np.arange(-r_max, r_max + 1)
    # kx fastest, like the reference's _hr.dat ordering by sorted tuples
    z, y, x = np.meshgrid(rng, rng, rng, indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float64)


def random_tb_model(n_wf: int = 8, r_max: int = 1, decay: float = 1.0, seed: int = 0,
                    with_r: bool = True, tb_convention: bool = True, a_bohr: float = 5.0,
                    soc_ev: float = 0.1, r_sigma_ang: float = 0.05,
                    kubo_tol: float = 1e-5) -> TBModel:
    """Seeded random TB model (see module docstring for the recipe)."""
    if n_wf % 2:
        raise ValueError("n_wf must be even (orbitals x spin)")
    rng = np.random.default_rng(seed)
    n_orb = n_wf // 2
    R = _cube(r_max)
    nR = R.shape[0]
    idx = {tuple(int(v) for v in R[i]): i for i in range(nR)}
    H = np.zeros((nR, n_wf, n_wf), np.complex128)
    r = np.zeros((nR, 3, n_wf, n_wf), np.complex128) if with_r else None
    sz = np.concatenate([np.ones(n_orb), -np.ones(n_orb)])
    for i in range(nR):
        key = tuple(int(v) for v in R[i])
        neg = tuple(-v for v in key)
        j = idx[neg]
        if key > neg:
            continue  # filled from its partner
        norm = float(np.sqrt(np.dot(R[i], R[i])))
        amp = np.exp(-norm / decay)
        X = (rng.standard_normal((n_wf, n_wf)) + 1j * rng.standard_normal((n_wf, n_wf))) * amp
        if abs(norm - 1.0) < 1e-12:
            X = X + 1j * soc_ev * np.diag(sz)
        if with_r:
            Y = (rng.standard_normal((3, n_wf, n_wf)) + 1j * rng.standard_normal((3, n_wf, n_wf))) * r_sigma_ang
        if i == j:  # R = 0: Hermitian with onsite energies
            X = 0.5 * (X + X.conj().T)
            X[np.diag_indices(n_wf)] = rng.uniform(-2.0, 2.0, n_wf)
            H[i] = X
            if with_r:
                r[i] = 0.5 * (Y + np.conj(np.swapaxes(Y, 1, 2)))
        else:
            H[i] = X
            H[j] = X.conj().T
            if with_r:
                r[i] = Y
                r[j] = np.conj(np.swapaxes(Y, 1, 2))
    tau = None
    if tb_convention:
        sites = np.array([_SITES[o % 4] + 0.125 * (o // 4) for o in range(n_orb)])
        tau = np.concatenate([sites, sites], axis=0) % 1.0
    return TBModel(R_frac=R, H=H / AU_TO_EV, r=None if r is None else r / AU_TO_ANGSTROM,
                   wf_centers=tau, a_latt=a_bohr * np.eye(3), kubo_tol=kubo_tol)


def bloch_hamiltonian(model: TBModel, kpts: np.ndarray) -> np.ndarray:
    """H(k) (nk, N, N) of a model in its own phase convention (numpy; used to
    place the near-crossings of :func:`near_crossing_model`)."""
    kpts = np.atleast_2d(np.asarray(kpts, np.float64))
    Hk = np.einsum("kr,rnm->knm", np.exp(2j * np.pi * kpts @ model.R_frac.T), model.H)
    if model.wf_centers is not None:
        d = model.wf_centers[None, :, :] - model.wf_centers[:, None, :]          # tau_m - tau_n at [n, m]
        Hk = Hk * np.exp(2j * np.pi * np.einsum("ka,nma->knm", kpts, d))
    return Hk


def _r0_phase(model: TBModel, k0: np.ndarray) -> np.ndarray:
    """exp(2 pi i k0.(tau_m - tau_n)): how H(R=0) enters H(k0)."""
    if model.wf_centers is None:
        return np.ones((model.n_wf, model.n_wf), np.complex128)
    d = model.wf_centers[None, :, :] - model.wf_centers[:, None, :]
    return np.exp(2j * np.pi * d @ k0)


def near_crossing_model(n_wf: int = 16, r_max: int = 2, decay: float = 1.5, seed: int = 4,
                        gaps_ev=(1e-3, 2e-3, 3.5e-3, 5e-3), ef_ev: float = 0.0, n_scan: int = 20,
                        min_sep: float = 0.2, sweeps: int = 12):
    """A random model (:func:`random_tb_model`) with len(gaps_ev) seeded
    near-crossings: at k-points k_j where the gap between bands N/2-1 and N/2
    has a local minimum, that gap is lowered to gaps_ev[j] and centred on the
    Fermi energy ef_ev.

    The k_j are the deepest local minima of that gap on an n_scan^3 mesh, at
    least ``min_sep`` apart, among those where ef_ev already lies between the
    two bands.  At each k_j a Hermitian change of H(R=0) acts in k-space as
    X_j = alpha (|c><c| - |v><v|) + beta (|c><c| + |v><v|) on the two band
    states there, which moves their energies to ef -+ gap/2 and leaves the
    other states at k_j untouched.  The changes for different k_j disturb one
    another slightly, so they are repeated until every gap is met.

    Returns (model, info) with info = {"k": (n, 3), "gap_ev": achieved gaps}.
    """
    model = random_tb_model(n_wf=n_wf, r_max=r_max, decay=decay, seed=seed)
    nv = n_wf // 2
    ef = ef_ev / AU_TO_EV
    q = (2.0 * np.arange(1, n_scan + 1) - n_scan - 1) / (2.0 * n_scan)
    kz, ky, kx = np.meshgrid(q, q, q, indexing="ij")
    grid = np.stack([kx.ravel(), ky.ravel(), kz.ravel()], axis=1)
    E = np.linalg.eigvalsh(bloch_hamiltonian(model, grid))
    gap = (E[:, nv] - E[:, nv - 1]).reshape(n_scan, n_scan, n_scan)
    inside = ((E[:, nv - 1] < ef) & (E[:, nv] > ef)).reshape(gap.shape)
    is_min = inside.copy()
    for ax in range(3):
        for sh in (-1, 1):
            is_min &= gap <= np.roll(gap, sh, axis=ax)
    cand = np.argsort(np.where(is_min, gap, np.inf).ravel())
    chosen = []
    for c in cand:
        if not is_min.ravel()[c]:
            break
        k = grid[c]
        dk = np.array([np.abs(((k - o) + 0.5) % 1.0 - 0.5).max() for o in chosen]) if chosen else np.array([1.0])
        if dk.min() >= min_sep:
            chosen.append(k)
        if len(chosen) == len(gaps_ev):
            break
    if len(chosen) < len(gaps_ev):
        raise ValueError("not enough separated gap minima with ef inside the gap")
    H0 = int(np.argmin(np.abs(model.R_frac).sum(axis=1)))
    targets = np.asarray(gaps_ev, np.float64) / AU_TO_EV
    for _ in range(sweeps):
        worst = 0.0
        for k0, g in zip(chosen, targets):
            w, U = np.linalg.eigh(bloch_hamiltonian(model, k0)[0])
            v, c = U[:, nv - 1], U[:, nv]
            alpha = 0.5 * (g - (w[nv] - w[nv - 1]))
            beta = ef - 0.5 * (w[nv] + w[nv - 1])
            worst = max(worst, abs(w[nv] - w[nv - 1] - g), abs(0.5 * (w[nv] + w[nv - 1]) - ef))
            X = (alpha + beta) * np.outer(c, c.conj()) + (beta - alpha) * np.outer(v, v.conj())
            model.H[H0] += np.conj(_r0_phase(model, k0)) * X
        if worst < 1e-9 / AU_TO_EV:
            break
    achieved = []
    for k0 in chosen:
        w = np.linalg.eigvalsh(bloch_hamiltonian(model, k0)[0])
        achieved.append((w[nv] - w[nv - 1]) * AU_TO_EV)
    return model, {"k": np.asarray(chosen), "gap_ev": np.asarray(achieved)}


def batch_workload(n_models: int = 64, seed: int = 3):
    """The batched form's workload: n_models independent seeded models, each
    with nWf drawn from {4, 6, ..., 64}, an R shell radius from {1, 2, 3}
    (nR 27-343), a mesh edge from {32, 48, 64, 96}, and a sweep of 201 Fermi
    energies over [-1, 1] eV with 25 meV Fermi-Dirac smearing (T = 290.1 K).
    Returns a list of (TBModel, job dict)."""
    rng = np.random.default_rng(seed)
    out = []
    ef = np.linspace(-1.0, 1.0, 201) / AU_TO_EV
    for i in range(n_models):
        n_wf = 2 * int(rng.integers(2, 33))
        r_max = int(rng.integers(1, 4))
        edge = int(rng.choice([32, 48, 64, 96]))
        m = random_tb_model(n_wf=n_wf, r_max=r_max, decay=1.5, seed=1000 + i)
        job = dict(mp_grid=(edge, edge, edge), ef_lst=ef, T_kelvin=290.1, valence_bands=n_wf // 2)
        out.append((m, job))
    return out


# Workloads: the model, mesh and Fermi settings each benchmark configuration uses.
# Every workload runs the reference's AHE job in full: with do_ahc it also forms
# velo_ahc_tens and kubo_ohc_tens (src/core.f90:221-230), here at one photon
# energy hw = 0 with the 1 meV broadening of the plain configuration.
WORKLOADS = {
    # plain FP64 case: nWf=8, R in {-1,0,1}^3, 16^3 mesh, E_F = 0, T = 0
    "tb8_r1_k16": dict(model=dict(n_wf=8, r_max=1, decay=1.0, seed=1), mp_grid=(16, 16, 16),
                       ef_ev=[0.0], T_kelvin=0.0, valence_bands=4),
    # precision form at scale: nWf=32, R in {-3..3}^3, 128^3 mesh in 64K-k chunks
    "tb32_r3_k128": dict(model=dict(n_wf=32, r_max=3, decay=1.5, seed=2), mp_grid=(128, 128, 128),
                         ef_ev=[0.0], T_kelvin=0.0, valence_bands=16),
    # largest: nWf=64, R in {-4..4}^3, 256^3 mesh, 401 Fermi energies, 25 meV smearing
    "tb64_r4_k256": dict(model=dict(n_wf=64, r_max=4, decay=1.5, seed=5), mp_grid=(256, 256, 256),
                         ef_ev=list(np.linspace(-1.5, 1.5, 401)), T_kelvin=290.1, valence_bands=32),
}


def workload(name: str):
    """(TBModel, job dict) of a named workload; job energies in Hartree."""
    w = WORKLOADS[name]
    model = random_tb_model(**w["model"])
    job = dict(mp_grid=tuple(w["mp_grid"]), ef_lst=np.asarray(w["ef_ev"], np.float64) / AU_TO_EV,
               T_kelvin=float(w["T_kelvin"]), valence_bands=int(w["valence_bands"]),
               hw_lst=np.asarray(w.get("hw_ev", [0.0]), np.float64) / AU_TO_EV,
               eta_smr=float(w.get("eta_ev", 1e-3)) / AU_TO_EV)
    return model, job
