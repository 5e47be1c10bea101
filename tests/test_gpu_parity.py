"""GPU parity of the CUDA path (through the C ABI) against the CPU oracle.

Tolerances (the plain form is all-FP64 and must match the reference's
LAPACK-zheevd FP64 path):
  eigenvalues                 1e-10 relative to max |E|
  sigma_ab, MEP tensors       1e-8 relative to the largest entry of each tensor
The mixed form (separable Fourier sums from FP32 slabs with an FP64 H(k), FP32
Jacobi plus the FP64 residual refinement, FP32 per-k work with FP64 energies,
FP64 k-sums and an FP64 rerun of near-degenerate k-points) is held to 1e-6
relative on the k-summed tensors.  Its tensor-core Fourier path (used for k
lists off the mesh, forced here with MEPI_FT=tc) accumulates in FP32 inside the
tensor core and is held to TC_TOL.
"""
import os

import numpy as np
import pytest

from mepinterp_gb300 import api
from mepinterp_gb300.generator import random_tb_model, workload
from oracle import ref_numpy as O

pytestmark = pytest.mark.gpu

KEYS = ["Ne_sum", "ahc", "mep_ic", "mep_lc", "mep_cs", "kubo_mep_ic", "kubo_mep_lc", "kubo_mep_cs"]
GOLD = os.path.join(os.path.dirname(__file__), "golden", "femn.npz")
E_TOL, SUM_TOL, MIXED_TOL = 1e-10, 1e-8, 1e-6
TC_TOL = 2e-5   # FP32 accumulation over K = 2 nR inside the tensor core
# The mixed form's Chern-Simons sums (mep_cs, kubo_mep_cs) on meshes or
# subsets of a few hundred to a few thousand k-points.  Each k-point carries
# FP32 noise of about 4e-7 of its own term (median; measured against the FP64
# path, unbiased in sign), and these sums cancel 20- to 50-fold across k
# (sum_k |t_k| / |sum_k t_k|), so on such samples the random walk of that noise
# is 6e-7 to 9e-7 of the sum and single draws reach 1.6e-6.  On the full 128^3
# mesh the walk averages out: test_mixed_full_mesh_partition holds every sum
# of the whole mesh to MIXED_TOL against the FP64 path.
MIXED_CS_TOL = 3e-6
CS_KEYS = ("mep_cs", "kubo_mep_cs")


def rel(a, b):
    """max |a - b| / max |b|, on complex arrays by the modulus of the complex
    difference (the imaginary parts count as much as the real ones)."""
    a, b = np.asarray(a), np.asarray(b)
    scale = np.abs(b).max()
    if scale == 0.0:
        return float(np.abs(a).max())
    return float(np.abs(a - b).max() / scale)


def check_sums(gpu, ref, tol, keys=KEYS):
    for k in keys:
        r = rel(gpu[k], ref[k])
        assert r < tol, f"{k}: rel err {r:.3e} (max |ref| {np.abs(ref[k]).max():.3e})"


def check_mixed(gpu, ref, keys=KEYS):
    """Mixed-form sums on a small mesh or a sampled subset: MIXED_TOL, the
    Chern-Simons sums MIXED_CS_TOL."""
    check_sums(gpu, ref, MIXED_TOL, keys=[k for k in keys if k not in CS_KEYS])
    check_sums(gpu, ref, MIXED_CS_TOL, keys=[k for k in keys if k in CS_KEYS])


def _check_complex(gpu, ref, tol, keys=("velo_ahc", "kubo_ohc")):
    for k in keys:
        scale = np.abs(ref[k]).max()
        r = float(np.abs(np.asarray(gpu[k]) - ref[k]).max() / scale)
        assert r < tol, f"{k}: rel err {r:.3e}"


@pytest.fixture(scope="module")
def model8():
    return random_tb_model(n_wf=8, r_max=1, seed=1)


def _check_per_k(model, kp, precision=api.PREC_FP64, e_tol=E_TOL, v_tol=1e-9, batch=64):
    """Per-k results of get_wann_interp against the oracle.  Eigenvectors carry
    a free phase per band (and a free basis in degenerate subspaces), so only
    gauge-invariant quantities are compared: the energies, |V|, the band
    diagonals of V, A and Omega, and the products P_ij(n,m) = V_i(n,m) V_j(m,n),
    real AND imaginary parts (the AHC is built from Im P, src/kubo.f90:65)."""
    with api.Context(model) as ctx:
        E, V, A, Om = ctx.get_wann_interp(kp, precision=precision)
    N = model.n_wf
    idx = np.arange(N)
    for s in range(0, kp.shape[0], batch):
        sl = slice(s, s + batch)
        E2, _U2, V2, A2, Om2 = O.interp_k(model.as_dict(), kp[sl])
        assert np.abs(E[sl] - E2).max() <= e_tol * np.abs(E2).max()
        assert rel(np.abs(V[sl]), np.abs(V2)) < v_tol
        assert rel(V[sl][:, :, idx, idx], V2[:, :, idx, idx]) < v_tol
        if A2 is not None:
            assert rel(A[sl], A2[:, :, idx, idx]) < v_tol
            assert rel(Om[sl], Om2[:, :, :, idx, idx]) < v_tol
        P = np.einsum("kinm,kjmn->kijnm", V[sl], V[sl])
        P2 = np.einsum("kinm,kjmn->kijnm", V2, V2)
        assert np.iscomplexobj(P) and np.abs(P2.imag).max() > 0
        assert rel(P, P2) < v_tol
        assert rel(P.imag, P2.imag) < v_tol


def test_eigenvalues_fp64(gpu_lib, model8):
    rng = np.random.default_rng(0)
    kp = rng.uniform(-0.5, 0.5, size=(97, 3))
    _check_per_k(model8, kp)


@pytest.mark.parametrize("n_wf,r_max", [(32, 3), (64, 2)])
def test_eigenvalues_fp64_large_n(gpu_lib, n_wf, r_max):
    """Per-k eigenvalue parity at 1e-10 at the headline band count (32) and at
    the largest supported one (64), with the gauge-invariant velocity checks."""
    m = random_tb_model(n_wf=n_wf, r_max=r_max, decay=1.5, seed=5 + n_wf)
    kp = np.random.default_rng(n_wf).uniform(-0.5, 0.5, size=(40, 3))
    _check_per_k(m, kp, batch=8)


@pytest.mark.parametrize("rot", ["tc", "simt"])
def test_per_k_mixed_nwf32(gpu_lib, monkeypatch, rot):
    """Per-k results of the mixed form at N = 32 (FP32 per-k work, refined FP64
    energies) against the oracle, with the tensor-core rotation (default) and
    the CUDA-core one (MEPI_ROT=simt): energies within 1e-9 of max |E|, the
    gauge-invariant velocity quantities within 2e-5 of their largest entry."""
    if rot == "simt":
        monkeypatch.setenv("MEPI_ROT", "simt")
    m = random_tb_model(n_wf=32, r_max=3, decay=1.5, seed=37)
    kp = np.random.default_rng(3).uniform(-0.5, 0.5, size=(48, 3))
    _check_per_k(m, kp, precision=api.PREC_MIXED, e_tol=1e-9, v_tol=2e-5, batch=8)


def test_rotation_tc_matches_simt_sums(gpu_lib, monkeypatch):
    """The tensor-core rotation (exact-slice FP16 digit products) and the
    CUDA-core one (Dot2 velocity blocks, FP32 connection and curvature) both
    give mixed-form sums within 1e-6 of the oracle on a 6^3 mesh of an N = 32
    model."""
    m = random_tb_model(n_wf=32, r_max=2, decay=1.5, seed=41)
    job = dict(mp_grid=(6, 6, 6), ef_lst=np.array([-0.01, 0.0, 0.01]), T_kelvin=300.0, valence_bands=16,
               hw_lst=np.array([0.0, 0.01]), eta_smr=0.002)
    tc = api.run(m, job, precision=api.PREC_MIXED)
    monkeypatch.setenv("MEPI_ROT", "simt")
    simt = api.run(m, job, precision=api.PREC_MIXED)
    ref = O.run(m.as_dict(), job, batch=36)
    check_mixed(tc, ref)
    check_mixed(simt, ref)
    _check_complex(tc, ref, MIXED_TOL)


@pytest.mark.parametrize("with_r,tb,gauge,sem,cart", [
    (True, True, True, "ref", False), (False, True, True, "ref", False), (True, False, True, "ref", False),
    (True, True, False, "ref", False), (True, True, True, "paper", False), (True, True, True, "ref", True),
])
def test_kloop_fp64_modes(gpu_lib, with_r, tb, gauge, sem, cart):
    m = random_tb_model(n_wf=8, r_max=1, seed=11, with_r=with_r, tb_convention=tb)
    m.semantics, m.do_gauge_trafo, m.use_cart_velo = sem, gauge, cart
    if cart:
        m.a_latt = np.array([[5.0, 0.2, 0.1], [0.3, 4.5, 0.0], [0.1, 0.2, 6.0]])
    job = dict(mp_grid=(6, 6, 6), ef_lst=np.array([-0.03, 0.0, 0.02]), T_kelvin=300.0, valence_bands=4)
    ref = O.run(m.as_dict(), job)
    got = api.run(m, job, precision=api.PREC_FP64)
    assert got["n_k"] == ref["n_k"] == 216
    check_sums(got, ref, SUM_TOL)


def test_kloop_fp64_config1(gpu_lib):
    """nWf=8, nR=27, 16^3 mesh, E_F=0, T=0 (the CPU-runnable configuration)."""
    model, job = workload("tb8_r1_k16")
    ref = O.run(model.as_dict(), job, batch=512)
    got = api.run(model, job, precision=api.PREC_FP64, chunk_k=1000)
    assert got["n_k"] == 4096
    check_sums(got, ref, SUM_TOL)
    _check_complex(got, ref, SUM_TOL)


def test_kloop_fp64_nwf32_subset(gpu_lib):
    """nWf=32, nR=343 model on a strided k subset of its 128^3 mesh."""
    model, job = workload("tb32_r3_k128")
    nk = 128 ** 3
    stride = nk // 96 + 1
    kidx = np.arange(0, nk, stride)
    ref = O.run(model.as_dict(), job, k_indices=kidx, batch=16)
    got = api.run(model, job, precision=api.PREC_FP64, k_begin=0, k_stride=stride)
    assert got["n_k"] == kidx.size
    check_sums(got, ref, SUM_TOL)


def test_fermi_sweep_finite_T(gpu_lib):
    m = random_tb_model(n_wf=12, r_max=2, decay=1.2, seed=21)
    ef = np.linspace(-1.0, 1.0, 37) / O.AU_TO_EV
    job = dict(mp_grid=(5, 5, 5), ef_lst=ef, T_kelvin=290.1, valence_bands=6)
    ref = O.run(m.as_dict(), job)
    got = api.run(m, job, precision=api.PREC_FP64)
    check_sums(got, ref, SUM_TOL)
    # the >= 64 Fermi-energy code path
    ef2 = np.linspace(-1.5, 1.5, 101) / O.AU_TO_EV
    job2 = dict(job, ef_lst=ef2)
    check_sums(api.run(m, job2, precision=api.PREC_FP64), O.run(m.as_dict(), job2), SUM_TOL)


@pytest.mark.parametrize("n_wf", [5, 16, 64])
def test_odd_and_large_n(gpu_lib, n_wf):
    m = random_tb_model(n_wf=n_wf + (n_wf % 2), r_max=1, seed=n_wf)
    if n_wf % 2:  # odd band count: drop the last orbital
        m.H = m.H[:, :n_wf, :n_wf]
        m.r = m.r[:, :, :n_wf, :n_wf]
        m.wf_centers = m.wf_centers[:n_wf]
    job = dict(mp_grid=(3, 3, 3), ef_lst=[0.0], T_kelvin=0.0, valence_bands=n_wf // 2)
    ref = O.run(m.as_dict(), job, batch=9)
    got = api.run(m, job, precision=api.PREC_FP64)
    check_sums(got, ref, SUM_TOL)
    mixed = api.run(m, job, precision=api.PREC_MIXED)
    check_mixed(mixed, ref)


def test_femn_golden_gpu(gpu_lib):
    g = np.load(GOLD)
    m = api.TBModel(R_frac=g["R_0p900"].astype(float), H=g["H_eV_0p900"] / O.AU_TO_EV,
                    wf_centers=g["wf_centers"], a_latt=g["latt_0p900"])
    job = dict(mp_grid=(32, 32, 32), ef_lst=[0.0], T_kelvin=0.0, valence_bands=4, do_mep=False, do_kubo=False)
    got = api.run(m, job, precision=api.PREC_FP64)
    _, vol = O.recip_latt(g["latt_0p900"])
    s = got["ahc"][:, :, 0] / abs(vol * 32 ** 3)
    gold = g["ahc_0p900"]
    assert abs(s[0, 1] - gold[0, 1]) < 2e-3 * abs(gold[0, 1])
    ref = O.run(dict(R_frac=m.R_frac, H=m.H, wf_centers=m.wf_centers, a_latt=m.a_latt), job, batch=1024)
    check_sums(got, ref, SUM_TOL, keys=["ahc", "Ne_sum"])


def test_k_partition_gpu(gpu_lib, model8):
    job = dict(mp_grid=(8, 8, 8), ef_lst=[0.0], T_kelvin=0.0, valence_bands=4)
    with api.Context(model8) as ctx:
        full = ctx.core_worker_loc(job)
        parts = [ctx.core_worker_loc(job, k_begin=r, k_stride=3) for r in range(3)]
    assert sum(p["n_k"] for p in parts) == 512
    for k in KEYS:
        assert rel(sum(p[k] for p in parts), full[k]) < 1e-12


def test_mixed_config1(gpu_lib):
    model, job = workload("tb8_r1_k16")
    ref = O.run(model.as_dict(), job, batch=512)
    got = api.run(model, job, precision=api.PREC_MIXED)
    assert got["n_k"] == 4096
    check_mixed(got, ref)
    _check_complex(got, ref, MIXED_TOL)


def test_mixed_fermi_sweep(gpu_lib):
    m = random_tb_model(n_wf=12, r_max=2, decay=1.2, seed=21)
    ef = np.linspace(-1.0, 1.0, 37) / O.AU_TO_EV
    job = dict(mp_grid=(6, 6, 6), ef_lst=ef, T_kelvin=290.1, valence_bands=6)
    ref = O.run(m.as_dict(), job)
    got = api.run(m, job, precision=api.PREC_MIXED)
    check_mixed(got, ref)


def test_mixed_full_mesh_partition(gpu_lib):
    """nWf=32 model on its full 128^3 mesh in the mixed form: every sum of the
    whole mesh within 1e-6 of the FP64 path on the same mesh (the accuracy
    target of the mixed form), two round-robin 'ranks' sum to the single run
    (size-independent property), and a strided subset agrees with the FP64
    path."""
    model, job = workload("tb32_r3_k128")
    with api.Context(model) as ctx:
        full = ctx.core_worker_loc(job, precision=api.PREC_MIXED)
        assert full["n_k"] == 128 ** 3
        full64 = ctx.core_worker_loc(job, precision=api.PREC_FP64)
        check_sums(full, full64, MIXED_TOL)
        _check_complex(full, full64, MIXED_TOL)
        parts = [ctx.core_worker_loc(job, precision=api.PREC_MIXED, k_begin=r, k_stride=2) for r in range(2)]
        for k in KEYS:
            assert rel(parts[0][k] + parts[1][k], full[k]) < 1e-9, k
        stride = 997
        a = ctx.core_worker_loc(job, precision=api.PREC_MIXED, k_stride=stride)
        b = ctx.core_worker_loc(job, precision=api.PREC_FP64, k_stride=stride)
        check_mixed(a, b)


def test_mixed_config2_subset_vs_oracle(gpu_lib):
    """The mixed form on a strided ~2,000-k subset of the nWf=32, nR=343, 128^3
    workload against the C oracle directly (not through the FP64 GPU path):
    every summed tensor, the optical Hall tensors included, within 1e-6."""
    from oracle import ref_c
    model, job = workload("tb32_r3_k128")
    stride = 1049
    ref = ref_c.run(model.as_dict(), job, k_begin=0, k_stride=stride)
    got = api.run(model, job, precision=api.PREC_MIXED, k_begin=0, k_stride=stride)
    assert got["n_k"] == ref["n_k"] == (128 ** 3 + stride - 1) // stride
    check_mixed(got, ref)
    _check_complex(got, ref, MIXED_TOL)


def _wide_r_model():
    """A model whose R box is wider than the separable sums take (|Rx| = 20)."""
    m = random_tb_model(n_wf=8, r_max=1, seed=3)
    n = m.n_wf
    rng = np.random.default_rng(3)
    t = 1e-3 * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    rr = 1e-3 * (rng.normal(size=(3, n, n)) + 1j * rng.normal(size=(3, n, n)))
    m.R_frac = np.vstack([m.R_frac, [[20.0, 0.0, 0.0], [-20.0, 0.0, 0.0]]])
    m.H = np.concatenate([m.H, t[None], t.conj().T[None]])
    m.r = np.concatenate([m.r, rr[None], np.conj(np.transpose(rr, (0, 2, 1)))[None]])
    return m


@pytest.mark.parametrize("case", ["tb", "wannier", "no_r", "wide_R"])
def test_fourier_paths_fp64(gpu_lib, monkeypatch, case):
    """The separable sums (default on a mesh) and the direct SIMT sums give the
    same FP64 results, and both match the oracle; a model whose R box is too
    wide for the separable form falls back to the direct sums."""
    if case == "wide_R":
        m = _wide_r_model()
    else:
        m = random_tb_model(n_wf=8, r_max=1, seed=7, with_r=(case != "no_r"), tb_convention=(case == "tb"))
    job = dict(mp_grid=(6, 5, 4), ef_lst=np.array([-0.02, 0.0]), T_kelvin=0.0, valence_bands=4)
    ref = O.run(m.as_dict(), job)
    sep = api.run(m, job, precision=api.PREC_FP64)
    monkeypatch.setenv("MEPI_FT", "simt")
    simt = api.run(m, job, precision=api.PREC_FP64)
    check_sums(sep, ref, SUM_TOL)
    check_sums(simt, ref, SUM_TOL)
    check_sums(sep, simt, 1e-10)


def test_mixed_tensor_core_fourier(gpu_lib, monkeypatch):
    model, job = workload("tb8_r1_k16")
    ref = O.run(model.as_dict(), job, batch=512)
    monkeypatch.setenv("MEPI_FT", "tc")
    got = api.run(model, job, precision=api.PREC_MIXED)
    check_sums(got, ref, TC_TOL)


def test_mixed_partial_ownership(gpu_lib):
    """A rank's share (k_begin, k_stride, k_count) walked in column order by the
    separable sums covers exactly the oracle's k-points."""
    m = random_tb_model(n_wf=10, r_max=2, decay=1.2, seed=9)
    job = dict(mp_grid=(7, 6, 5), ef_lst=np.array([0.0]), T_kelvin=0.0, valence_bands=5)
    kidx = 2 + 3 * np.arange(61)
    ref = O.run(m.as_dict(), job, k_indices=kidx)
    got = api.run(m, job, precision=api.PREC_MIXED, k_begin=2, k_stride=3, k_count=61)
    assert got["n_k"] == 61
    check_mixed(got, ref)
    got64 = api.run(m, job, precision=api.PREC_FP64, k_begin=2, k_stride=3, k_count=61)
    check_sums(got64, ref, SUM_TOL)


@pytest.mark.parametrize("precision", [api.PREC_FP64, api.PREC_MIXED])
def test_separable_slabs_under_memory_limit(gpu_lib, precision):
    """Under a 2 MiB device-memory limit the separable sums of a 9x6x5 mesh are
    built for a few qx at a time during the run (extra Fourier stages beyond
    one per chunk); the sums match the oracle and the unlimited run."""
    m = random_tb_model(n_wf=8, r_max=1, seed=21)
    job = dict(mp_grid=(9, 6, 5), ef_lst=np.array([-0.01, 0.0, 0.02]), T_kelvin=0.0, valence_bands=4,
               hw_lst=np.array([0.0, 0.02]), eta_smr=0.002)
    ref = O.run(m.as_dict(), job)
    with api.Context(m) as ctx:
        free = ctx.core_worker_loc(job, precision=precision)
        ctx.set_mem_limit(2 << 20)
        lim = ctx.core_worker_loc(job, precision=precision)
        t = ctx.timing()
        assert t["ft_launches"] > t["eig_launches"], t
        ctx.set_mem_limit(0)
        again = ctx.core_worker_loc(job, precision=precision)
    if precision == api.PREC_FP64:
        check_sums(lim, ref, SUM_TOL)
        _check_complex(lim, ref, SUM_TOL)
        # only the chunk boundaries move, so the sums agree to rounding
        check_sums(lim, free, 1e-12)
        check_sums(again, free, 1e-12)
    else:
        # the mixed form's FP32 sums group the k-points of a CTA differently
        check_mixed(lim, ref)
        _check_complex(lim, ref, MIXED_TOL)
        check_mixed(lim, free)
        check_mixed(again, free)


@pytest.mark.parametrize("T_kelvin,n_ef", [(0.0, 5), (290.1, 70)])
def test_optical_hall_tensors(gpu_lib, T_kelvin, n_ef):
    """velo_ahc_tens and kubo_ohc_tens (src/kubo.f90:86-198) over a photon-energy
    list and a Fermi sweep (70 energies span several occupation tiles), both
    forms against the oracle."""
    m = random_tb_model(n_wf=10, r_max=2, decay=1.2, seed=17)
    job = dict(mp_grid=(5, 4, 6), ef_lst=np.linspace(-0.02, 0.02, n_ef), T_kelvin=T_kelvin, valence_bands=5,
               hw_lst=np.linspace(0.0, 0.03, 4), eta_smr=0.002)
    ref = O.run(m.as_dict(), job)
    got = api.run(m, job, precision=api.PREC_FP64)
    _check_complex(got, ref, SUM_TOL)
    check_sums(got, ref, SUM_TOL)
    mixed = api.run(m, job, precision=api.PREC_MIXED)
    _check_complex(mixed, ref, MIXED_TOL)


def test_run_argument_errors(gpu_lib, model8):
    with api.Context(model8) as ctx:
        with pytest.raises(api.MepiError) as e:
            ctx.core_worker_loc(dict(mp_grid=(0, 4, 4), ef_lst=[0.0], valence_bands=4))
        assert e.value.status == api.ERR_ARG
        with pytest.raises(api.MepiError) as e:
            ctx.core_worker_loc(dict(mp_grid=(4, 4, 4), ef_lst=[0.0], valence_bands=9))
        assert e.value.status == api.ERR_ARG
        with pytest.raises(api.MepiError) as e:
            ctx.core_worker_loc(dict(mp_grid=(4, 4, 4), ef_lst=[np.nan], valence_bands=4))
        assert e.value.status == api.ERR_ARG
        # still usable after rejected calls
        ok = ctx.core_worker_loc(dict(mp_grid=(2, 2, 2), ef_lst=[0.0], valence_bands=4))
        assert ok["n_k"] == 8
