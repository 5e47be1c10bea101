"""CPU oracle (numpy) for MEPinterp's per-k-point Wannier-interpolation path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it.  The product path (``mepinterp_gb300`` and its CUDA library) never calls
into it and fails loudly when its CUDA library is missing.

It restates the reference algorithm in FP64/complex128, vectorised over a batch
of k-points, following (file:line within cMax347/MEPinterp):

* k-mesh ............ src/k_space.f90:341-375 (get_kpt_idx / get_rel_kpt),
                      src/core.f90:165-178 (loop order kz > ky > kx)
* Fourier sums ...... src/wann_interp.f90:151-384 (FT_R_to_k, both the
                      tight-binding and the Wannier phase convention)
* eigensolve ........ src/matrix_math.f90:192-226 (zheevd_wrapper, jobz=V,
                      uplo=U); numpy.linalg.eigh calls LAPACK ?heevd
* gauge rotation .... src/wann_interp.f90:465-658 (rotate_gauge,
                      get_gauge_covar_deriv, conn_gaugeTrafo, curv_gaugeTrafo)
* velocity .......... src/wann_interp.f90:406-444 (get_velo)
* occupations ....... src/statistics.f90:41-124 (fd_stat, fd_get_N_el)
* AHC ............... src/kubo.f90:37-78 (kubo_ahc_tens)
* optical Hall ...... src/kubo.f90:86-198 (velo_ahc_tens, kubo_ohc_tens)
* Niu MEP ........... src/mep_niu.f90:20-159 (mep_niu_CS / _LC / _IC)
* Kubo MEP .......... src/kubo_mep.f90:16-149 (kubo_mep_CS / _LC / _IC)
* k-sum, Fermi pick,
  normalisation ..... src/core.f90:317-603, src/k_space.f90:81-202

Positions this restatement takes where the reference is not reproducible
(the CUDA path takes the same ones):

* D1  rotate_gauge rotates the connection from a stale buffer
      (src/wann_interp.f90:525-535); here A_bar = U^dag A^W U.
* D2  get_velo never writes V_nn when r(R) is present
      (src/wann_interp.f90:427-437); here V_nn = Hbar_a(n,n).
* D3  zgemm receives real alpha/beta (src/matrix_math.f90:651); here 1 and 0.
* D4/D5 (curvature and velocity built from A^H = A_bar + iD) are replicated in
  semantics ``"ref"``; semantics ``"paper"`` uses A_bar instead.
* D11 get_kpt_idx strides (src/k_space.f90:345) are replaced by the
  row-major formula; identical on the cubic meshes used here.
"""
from __future__ import annotations

import numpy as np

# src/constants.f90:13-22
PI = 4.0 * np.arctan(1.0)
AU_TO_EV = 27.211385
AU_TO_ANGSTROM = 0.52917721092
KB_EH_K = 8.6173303e-5 / AU_TO_EV
MIN_TEMP = 1e-2  # src/statistics.f90:32


def levi_civita() -> np.ndarray:
    """src/matrix_math.f90:125-139."""
    e = np.zeros((3, 3, 3))
    e[0, 1, 2] = e[1, 2, 0] = e[2, 0, 1] = 1.0
    e[0, 2, 1] = e[2, 1, 0] = e[1, 0, 2] = -1.0
    return e


LEVI = levi_civita()


# --------------------------------------------------------------------------
# k-space
# --------------------------------------------------------------------------
def rel_kpts(mp_grid, k_index: np.ndarray) -> np.ndarray:
    """Monkhorst-Pack points for 0-based linear indices (kx fastest).

    src/k_space.f90:351-375: k_i = (2 q_i - n_i - 1) / (2 n_i), q_i 1-based.
    src/core.f90:165-170: loop kz > ky > kx, so kx is the fastest index.
    """
    n1, n2, n3 = (int(x) for x in mp_grid)
    k_index = np.asarray(k_index, dtype=np.int64)
    qx = k_index % n1 + 1
    qy = (k_index // n1) % n2 + 1
    qz = k_index // (n1 * n2) + 1
    out = np.empty((k_index.size, 3))
    for col, q, n in ((0, qx, n1), (1, qy, n2), (2, qz, n3)):
        out[:, col] = (2.0 * q.astype(np.float64) - float(n) - 1.0) / (2.0 * float(n))
    return out


def recip_latt(a_latt: np.ndarray):
    """src/k_space.f90:263-292 (columns of a_latt are used as a1, a2, a3)."""
    a1, a2, a3 = a_latt[:, 0], a_latt[:, 1], a_latt[:, 2]
    unit_vol = float(np.dot(np.cross(a1, a2), a3))
    b = np.empty((3, 3))
    b[:, 0] = 2.0 * PI * np.cross(a2, a3) / unit_vol
    b[:, 1] = 2.0 * PI * np.cross(a3, a1) / unit_vol
    b[:, 2] = 2.0 * PI * np.cross(a1, a2) / unit_vol
    return b, unit_vol


# --------------------------------------------------------------------------
# Fourier sums (W gauge)
# --------------------------------------------------------------------------
def ft_R_to_k(model: dict, kpts: np.ndarray):
    """Return H, H_a, A_a, Om_ab in the Wannier gauge for each k.

    src/wann_interp.f90:151-384.  Shapes: H (nk,N,N), Ha (nk,3,N,N),
    A (nk,3,N,N) or None, Om (nk,3,3,N,N) or None.
    The per-element phase angle is computed exactly as in the reference loop
    (one angle per (R, n, m) in the tight-binding convention).
    """
    R = np.asarray(model["R_frac"], dtype=np.float64)          # (nR,3)
    H_R = np.asarray(model["H"], dtype=np.complex128)          # (nR,N,N)
    r_R = model.get("r")                                      # (nR,3,N,N) | None
    tau = model.get("wf_centers")                             # (N,3) | None
    a_latt = np.asarray(model["a_latt"], dtype=np.float64)
    cart = bool(model.get("use_cart_velo", False))
    nk = kpts.shape[0]
    N = H_R.shape[1]
    two_pi = 2.0 * PI
    b_latt, _ = recip_latt(a_latt)

    if tau is not None:
        tau = np.asarray(tau, dtype=np.float64)
        # delta_at(:,n,m) = atom_frac(:,m) - atom_frac(:,n)   (:200-205)
        dtau = tau[None, :, :] - tau[:, None, :]               # (n,m,3)
        dR = R[:, None, None, :] + dtau[None]                  # (nR,n,m,3)
    else:
        dR = np.broadcast_to(R[:, None, None, :], (R.shape[0], N, N, 3))

    # derivative weights dR_cart (:216, :231-233, :267-271, :310-314)
    if cart:
        dRc = np.einsum("ij,rnmj->rnmi", a_latt, dR)
    else:
        dRc = two_pi * dR

    # phase angles
    if tau is not None and cart:
        kc = kpts @ b_latt.T                                  # matmul(recip_latt,kpt)
        ang_H = np.einsum("ki,rnmi->krnm", kc, dRc)           # (:216-217)
    else:
        ang_H = two_pi * np.einsum("ki,rnmi->krnm", kpts, dR)  # (:219, :259)
    ang_A = two_pi * np.einsum("ki,rnmi->krnm", kpts, dR)      # (:306, :348)

    ph_H = np.cos(ang_H) + 1j * np.sin(ang_H)
    H = np.einsum("krnm,rnm->knm", ph_H, H_R)
    Ha = 1j * np.einsum("krnm,rnma,rnm->kanm", ph_H, dRc, H_R)

    A = Om = None
    if r_R is not None:
        r_R = np.asarray(r_R, dtype=np.complex128)
        ph_A = np.cos(ang_A) + 1j * np.sin(ang_A)
        A = np.einsum("krnm,ranm->kanm", ph_A, r_R)
        # Om(a,b) += ph*i*dRc_a*r_b ; Om(a,b) -= ph*i*dRc_b*r_a   (:321-326)
        t = 1j * np.einsum("krnm,rnma,rbnm->kabnm", ph_A, dRc, r_R)
        Om = t - np.swapaxes(t, 1, 2)
    return H, Ha, A, Om


# --------------------------------------------------------------------------
# eigensolve + gauge transformation + velocity
# --------------------------------------------------------------------------
def zheevd(Hk: np.ndarray):
    """src/matrix_math.f90:192-226 (uplo='U'); eigenvalues ascending."""
    E, U = np.linalg.eigh(Hk, UPLO="U")
    return E, U


def _dag(X):
    return np.conj(np.swapaxes(X, -1, -2))


def _comm(X, Y):
    return X @ Y - Y @ X


def gauge_and_velocity(model: dict, E, U, Ha, A, Om):
    """src/wann_interp.f90:56-108 (after the FT), :406-658.

    Returns V (nk,3,N,N), A_out, Om_out (H-gauge connection/curvature, or the
    W-gauge ones without a gauge transformation; None without r(R)).
    """
    kubo_tol = float(model.get("kubo_tol", 1e-5))
    semantics = model.get("semantics", "ref")
    do_gauge = bool(model.get("do_gauge_trafo", True))
    Ud = _dag(U)[:, None]
    Uc = U[:, None]
    Abar = None
    if do_gauge:
        Hb = Ud @ Ha @ Uc                                      # :517-528
        if A is not None:
            Abar = Ud @ A @ Uc                                 # D1 fixed
            Omb = _dag(U)[:, None, None] @ Om @ U[:, None, None]  # :538-544
            dE = E[:, None, :] - E[:, :, None]                 # (k,n,m) = E_m - E_n
            with np.errstate(divide="ignore", invalid="ignore"):
                D = np.where(np.abs(dE)[:, None] > kubo_tol, Hb / dE[:, None], 0.0)
            N = E.shape[1]
            eye = np.eye(N, dtype=bool)
            D = np.where(eye[None, None], 0.0, D)              # :578-596 (n /= m only)
            AH = Abar + 1j * D                                 # :620-633
            Ause = AH if semantics == "ref" else Abar          # D4
            OmH = np.empty_like(Omb)
            for a in range(3):                                 # :645-654
                for b in range(3):
                    OmH[:, a, b] = (Omb[:, a, b] - _comm(D[:, a], Ause[:, b])
                                    + _comm(D[:, b], Ause[:, a])
                                    - 1j * _comm(D[:, a], D[:, b]))
            A_out, Om_out = AH, OmH
        else:
            A_out = Om_out = None
    else:
        Hb = Ha
        A_out, Om_out = A, Om
    if A_out is not None:
        Avel = A_out if (semantics == "ref" or not do_gauge) else Abar   # D5
        dE = E[:, None, :] - E[:, :, None]                     # E_q - E_p at (p,q)
        V = Hb - 1j * dE[:, None] * Avel                       # :427-436
        N = E.shape[1]
        idx = np.arange(N)
        V[:, :, idx, idx] = Hb[:, :, idx, idx]                 # D2 position
    else:
        V = Hb.copy()                                          # :439
    return V, A_out, Om_out


# --------------------------------------------------------------------------
# occupations
# --------------------------------------------------------------------------
def fd_stat(E: np.ndarray, ef_lst: np.ndarray, T_kelvin: float) -> np.ndarray:
    """src/statistics.f90:65-90 -> f[k, e, n]."""
    E = np.asarray(E)[:, None, :]
    ef = np.asarray(ef_lst, dtype=np.float64)[None, :, None]
    if T_kelvin > MIN_TEMP:
        T_smear = KB_EH_K * T_kelvin
        with np.errstate(over="ignore"):
            return 1.0 / (1.0 + np.exp((E - ef) / T_smear))
    return (E < ef).astype(np.float64)


# --------------------------------------------------------------------------
# band sums (per k, returned per k so callers can sum in any order)
# einsum letter z is the k batch; a,b,c,i,j,l are Cartesian; o = n0, n, m, p bands
# --------------------------------------------------------------------------
def kubo_ahc(E, V, f):
    """src/kubo.f90:37-78 -> (nk,3,3,n_eF)."""
    N = E.shape[1]
    dE = E[:, None, :] - E[:, :, None]                         # E_np - E_n at (n,np)
    off = ~np.eye(N, dtype=bool)
    with np.errstate(divide="ignore", invalid="ignore"):
        w = np.where(off[None], 1.0 / dE ** 2, 0.0)
    prod = np.einsum("zinp,zjpn->znpij", V, V)
    curv = -2.0 * np.einsum("znpij,znp->znij", prod.imag, w)
    return -np.einsum("znij,zen->zije", curv, f)


def _ic_sum(V, sel, w):
    """sum_{n,m} w[o,n,m] * (-sum_cl eps_jcl Re(V_i(o,n) V_c(n,m) V_l(m,o)))."""
    Vi = V[:, :, sel, :]                                        # (z,i,o,n)
    Vl = V[:, :, :, sel]                                        # (z,l,m,o)
    G = np.einsum("jcl,zcnm,zlmo->zjonm", LEVI, V, Vl)          # (z,j,o,n,m)
    return -np.einsum("zion,zjonm,zonm->zijo", Vi, G, w).real


def _lc_sum(V, sel, w3):
    """sum_n w3[o,n] * sum_cl eps_jcl Re(V_i(o,n) V_c(n,o) V_l(o,o))."""
    Vi = V[:, :, sel, :]                                        # (z,i,o,n)
    Vc = V[:, :, :, sel]                                        # (z,c,n,o)
    Vnn = V[:, :, sel, sel]                                     # (z,l,o)
    G = np.einsum("jcl,zcno,zlo->zjon", LEVI, Vc, Vnn)          # (z,j,o,n)
    return np.einsum("zion,zjon,zon->zijo", Vi, G, w3).real


def _cs_val(A, Om, sel):
    """0.5 Re(dot_product(A(:,o,o), om_vect)) per band (src/mep_niu.f90:35-37)."""
    om_vec = np.einsum("abc,zabo->zco", LEVI, Om[:, :, :, sel, sel])
    return 0.5 * np.einsum("zco,zco->zo", np.conj(A[:, :, sel, sel]), om_vec).real


def mep_niu(model, E, V, A, Om, n_val):
    """src/mep_niu.f90:20-159 -> ic, lc, cs each (nk,3,3,n_val)."""
    kubo_tol = float(model.get("kubo_tol", 1e-5))
    nk, _, N, _ = V.shape
    sel = np.arange(n_val)
    dn = E[:, sel, None] - E[:, None, :]                        # (z,o,n) = E0 - En
    # IC: den = (E0-En)^2 (E0-Em), skip n==n0, m==n0, |den|<=tol   (:129-132)
    den = dn[:, :, :, None] ** 2 * dn[:, :, None, :]
    mask = np.ones((n_val, N, N), dtype=bool)
    mask[sel, sel, :] = False
    mask[sel, :, sel] = False
    ok = mask[None] & (np.abs(den) > kubo_tol)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        w = np.where(ok, 1.0 / den, 0.0)
    ic = _ic_sum(V, sel, w)
    # LC: den = (E0-En)^3, skip n==n0, |den|<=tol   (:71-73)
    den3 = dn ** 3
    mask3 = np.ones((n_val, N), dtype=bool)
    mask3[sel, sel] = False
    ok3 = mask3[None] & (np.abs(den3) > kubo_tol)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        w3 = np.where(ok3, 1.0 / den3, 0.0)
    lc = _lc_sum(V, sel, w3)
    cs = np.zeros((nk, 3, 3, n_val))
    if A is not None and Om is not None:
        val = _cs_val(A, Om, sel)
        for i in range(3):
            cs[:, i, i, :] = val
    return ic, lc, cs


def kubo_mep(model, E, V, A, Om, f):
    """src/kubo_mep.f90:16-149 -> ic, lc, cs each (nk,3,3,n_eF); no kuboTol guard."""
    nk, _, N, _ = V.shape
    sel = np.arange(N)
    dn = E[:, :, None] - E[:, None, :]                          # (z,o,n) = E0 - En
    off = ~np.eye(N, dtype=bool)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        den = dn[:, :, None, :] * dn[:, :, :, None] ** 2        # (E0-Em)(E0-En)^2 at (o,n,m)
        mask = off[:, :, None] & off[:, None, :]
        w = np.where(mask[None], 1.0 / den, 0.0)
        w3 = np.where(off[None], 1.0 / dn ** 3, 0.0)
    icn = _ic_sum(V, sel, w)
    lcn = _lc_sum(V, sel, w3)
    ic = np.einsum("zijo,zeo->zije", icn, f)
    lc = np.einsum("zijo,zeo->zije", lcn, f)
    cs = np.zeros((nk, 3, 3, f.shape[1]))
    if A is not None and Om is not None:
        scal = np.einsum("zeo,zo->ze", f, _cs_val(A, Om, sel))
        for i in range(3):
            cs[:, i, i, :] = scal
    return ic, lc, cs


# --------------------------------------------------------------------------
# one batch of k-points through the whole path
# --------------------------------------------------------------------------
def interp_k(model: dict, kpts: np.ndarray):
    """get_wann_interp (src/wann_interp.f90:56-108) for a batch of k."""
    H, Ha, A, Om = ft_R_to_k(model, kpts)
    E, U = zheevd(H)
    V, A_out, Om_out = gauge_and_velocity(model, E, U, Ha, A, Om)
    return E, U, V, A_out, Om_out


def gap_at(E: np.ndarray, ef: float) -> np.ndarray:
    """E_c - E_v across ef per k (twice the distance to the nearest band when
    ef lies outside all bands)."""
    N = E.shape[1]
    nF = (E < ef).sum(axis=1)
    inner = np.clip(nF, 1, N - 1)
    rows = np.arange(E.shape[0])
    gap = E[rows, inner] - E[rows, inner - 1]
    gap = np.where(nF == 0, 2.0 * (E[:, 0] - ef), gap)
    return np.where(nF == N, 2.0 * (ef - E[:, -1]), gap)


def run(model: dict, job: dict, k_indices=None, batch: int = 64, perk: bool = False) -> dict:
    """Body of the k-loop, src/core.f90:165-270, summed over the given k.

    Returns the unnormalised local sums (the reference's *_loc arrays):
    Ne_sum (n_eF,), ahc (3,3,n_eF), mep_ic/lc/cs (3,3,n_val),
    kubo_mep_ic/lc/cs (3,3,n_eF), n_k; with job["hw_lst"] (Hartree) and
    do_ahc also velo_ahc and kubo_ohc (3,3,n_hw,n_eF) complex, smeared by
    i * job["eta_smr"] (src/input_paras.f90:181).  With ``perk`` also
    "perk" (n_k, 4): per k the (y,z), (z,x), (x,y) entries of its
    kubo_ahc_tens term at ef_lst[0] and the band gap across ef_lst[0].
    """
    mp = job["mp_grid"]
    nk_tot = int(mp[0]) * int(mp[1]) * int(mp[2])
    if k_indices is None:
        k_indices = np.arange(nk_tot, dtype=np.int64)
    ef = np.asarray(job["ef_lst"], dtype=np.float64)
    n_eF = ef.size
    n_val = int(job["valence_bands"])
    T = float(job.get("T_kelvin", 0.0))
    out = {
        "Ne_sum": np.zeros(n_eF), "ahc": np.zeros((3, 3, n_eF)),
        "mep_ic": np.zeros((3, 3, n_val)), "mep_lc": np.zeros((3, 3, n_val)),
        "mep_cs": np.zeros((3, 3, n_val)),
        "kubo_mep_ic": np.zeros((3, 3, n_eF)), "kubo_mep_lc": np.zeros((3, 3, n_eF)),
        "kubo_mep_cs": np.zeros((3, 3, n_eF)), "n_k": 0,
    }
    do_ahc = job.get("do_ahc", True)
    do_mep = job.get("do_mep", True)
    do_kubo = job.get("do_kubo", True)
    hw = job.get("hw_lst")
    do_omega = do_ahc and hw is not None and len(hw) > 0
    if do_omega:
        hw = np.asarray(hw, dtype=np.float64)
        eta = float(job.get("eta_smr", 0.0))
        out["velo_ahc"] = np.zeros((3, 3, hw.size, n_eF), complex)
        out["kubo_ohc"] = np.zeros((3, 3, hw.size, n_eF), complex)
    if perk:
        out["perk"] = np.zeros((len(k_indices), 4))
    for s in range(0, len(k_indices), batch):
        kidx = np.asarray(k_indices[s:s + batch])
        kpts = rel_kpts(mp, kidx)
        E, U, V, A, Om = interp_k(model, kpts)
        f = fd_stat(E, ef, T)                                   # (k,e,n)
        if perk:
            a = kubo_ahc(E, V, f[:, :1, :])[..., 0]             # (k,3,3) at ef_lst[0]
            out["perk"][s:s + kidx.size] = np.stack([a[:, 1, 2], a[:, 2, 0], a[:, 0, 1], gap_at(E, ef[0])], axis=1)
        out["Ne_sum"] += f.sum(axis=(0, 2))                     # :187
        if do_mep:
            ic, lc, cs = mep_niu(model, E, V, A, Om, n_val)
            out["mep_ic"] += ic.sum(0)
            out["mep_lc"] += lc.sum(0)
            out["mep_cs"] += cs.sum(0)
        if do_kubo:
            ic, lc, cs = kubo_mep(model, E, V, A, Om, f)
            out["kubo_mep_ic"] += ic.sum(0)
            out["kubo_mep_lc"] += lc.sum(0)
            out["kubo_mep_cs"] += cs.sum(0)
        if do_ahc:
            out["ahc"] += kubo_ahc(E, V, f).sum(0)
        if do_omega:
            out["velo_ahc"] += velo_ahc(E, V, f, hw, eta).sum(0)
            out["kubo_ohc"] += kubo_ohc(E, V, f, hw, eta).sum(0)
        out["n_k"] += kidx.size
    return out


def fermi_selector(n_k_glob: int, Ne_sum: np.ndarray, n_val: int) -> int:
    """src/core.f90:317-415: first index minimising |N_el(eF) - N_val| (0-based)."""
    Ne = np.asarray(Ne_sum, dtype=np.float64) / n_k_glob
    opt_idx, opt_err = 0, abs(Ne[0] - float(n_val))
    for i in range(Ne.size):
        err = abs(Ne[i] - float(n_val))
        if err < opt_err:
            opt_idx, opt_err = i, err
    return opt_idx


def integrate(loc: dict, mp_grid, a_latt, n_val: int) -> dict:
    """src/core.f90:419-603 + src/k_space.f90:81-202 on one rank."""
    _, unit_vol = recip_latt(np.asarray(a_latt, dtype=np.float64))
    nk = int(mp_grid[0]) * int(mp_grid[1]) * int(mp_grid[2])
    norm = abs(unit_vol * float(nk))
    e = fermi_selector(loc["n_k"], loc["Ne_sum"], n_val)
    res = {"eF_idx": e}
    res["mep_ic"] = loc["mep_ic"].sum(-1) / norm
    res["mep_lc"] = loc["mep_lc"].sum(-1) / norm
    res["mep_cs"] = loc["mep_cs"].sum(-1) / norm
    res["mep_tens"] = res["mep_ic"] + res["mep_lc"] + res["mep_cs"]
    res["mep_bands"] = (loc["mep_ic"] + loc["mep_lc"] + loc["mep_cs"]) / norm
    for key in ("kubo_mep_ic", "kubo_mep_lc", "kubo_mep_cs"):
        res[key] = loc[key][:, :, e] / norm
    res["kubo_mep_tens"] = res["kubo_mep_ic"] + res["kubo_mep_lc"] + res["kubo_mep_cs"]
    res["ahc_tens"] = loc["ahc"][:, :, e] / norm
    if "velo_ahc" in loc:                                       # :501-508
        res["ahc_velo"] = loc["velo_ahc"][:, :, :, e] / norm
        res["ohc_velo"] = loc["kubo_ohc"][:, :, :, e] / norm
    return res


def velo_ahc(E, V, f, hw_lst, eta):
    """velo_ahc_tens, src/kubo.f90:86-140, per k: (nk,3,3,n_hw,n_eF) complex,
        o(i,j,w,e) = sum_{n != n'} (f(e,n) - f(e,n')) Im(V_i(n,n') V_j(n',n))
                                  / ((E_n - E_n')^2 - (hw_w + i eta)^2)."""
    N = E.shape[1]
    off = ~np.eye(N, dtype=bool)
    dE2 = (E[:, :, None] - E[:, None, :]) ** 2                 # (k,n,n')
    z = (np.asarray(hw_lst, dtype=np.float64) + 1j * eta) ** 2
    with np.errstate(divide="ignore", invalid="ignore"):
        w = np.where(off[None, :, :, None], 1.0 / (dE2[..., None] - z), 0.0)   # (k,n,n',w)
    prod = np.einsum("kinp,kjpn->knpij", V, V).imag
    df = f[:, :, :, None] - f[:, :, None, :]                    # (k,e,n,n')
    return np.einsum("knpij,knpw,kenp->kijwe", prod, w, df)


def kubo_ohc(E, V, f, hw_lst, eta):
    """kubo_ohc_tens, src/kubo.f90:146-198, per k: (nk,3,3,n_hw,n_eF) complex,
        z(i,j,w,e) = sum_{m != n} i V_i(n,m) V_j(m,n) (f(e,m) - f(e,n))
                                  / ((E_m - E_n)(E_m - E_n - hw_w - i eta)),
    with no degeneracy guard (D9)."""
    N = E.shape[1]
    off = ~np.eye(N, dtype=bool)
    dE = E[:, None, :] - E[:, :, None]                         # (k,n,m) = E_m - E_n
    hw = np.asarray(hw_lst, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        w = np.where(off[None, :, :, None], 1.0 / (dE[..., None] * (dE[..., None] - hw - 1j * eta)), 0.0)
    prod = np.einsum("kinm,kjmn->knmij", V, V)
    df = f[:, :, None, :] - f[:, :, :, None]                    # (k,e,n,m) = f(e,m) - f(e,n)
    return 1j * np.einsum("knmij,knmw,kenm->kijwe", prod, w, df)


def velo_ahc_hw0(E, V, f, eta):
    """src/kubo.f90:86-140 at hbar*omega = 0 (cross-check for the fixtures)."""
    N = E.shape[1]
    dE2 = (E[:, :, None] - E[:, None, :]) ** 2                 # (n,np)
    off = ~np.eye(N, dtype=bool)
    den = dE2 - (1j * eta) ** 2
    prod = np.einsum("kinp,kjpn->knpij", V, V).imag
    df = f[:, :, :, None] - f[:, :, None, :]                    # (k,e,n,np)
    w = np.where(off[None], 1.0 / den, 0.0)
    return np.einsum("knpij,knp,kenp->kije", prod, w, df)
