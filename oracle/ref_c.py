"""ctypes front end of the C oracle (oracle/ref_c.c).

TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the product
never imports this module.  ``build()`` compiles ``ref_c.c`` with gcc into
``oracle/libmepi_oracle.so``; LAPACK ``zheevd`` comes from scipy's bundled
OpenBLAS (exported there as ``scipy_zheevd_``) or any host LAPACK exporting
``zheevd_``.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ref_c.c")
LIB = os.path.join(HERE, "libmepi_oracle.so")


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["gcc", "-O3", "-std=gnu11", "-fopenmp", "-fPIC", "-shared", SRC, "-o", LIB, "-lm"]
        subprocess.check_call(cmd)
    return LIB


class _Model(C.Structure):
    _fields_ = [("n_wf", C.c_int32), ("n_R", C.c_int32),
                ("R_frac", C.c_void_p), ("H", C.c_void_p), ("r", C.c_void_p),
                ("wf_centers", C.c_void_p), ("a_latt", C.c_double * 9),
                ("do_gauge_trafo", C.c_int32), ("use_cart_velo", C.c_int32),
                ("semantics", C.c_int32), ("kubo_tol", C.c_double)]


class _Job(C.Structure):
    _fields_ = [("mp_grid", C.c_int32 * 3), ("n_eF", C.c_int32), ("ef_lst", C.c_void_p),
                ("T_kelvin", C.c_double), ("valence_bands", C.c_int32),
                ("do_ahc", C.c_int32), ("do_mep", C.c_int32), ("do_kubo", C.c_int32),
                ("n_hw", C.c_int32), ("hw_lst", C.c_void_p), ("eta_smr", C.c_double)]


class _Out(C.Structure):
    _fields_ = [("Ne_sum", C.c_void_p), ("ahc", C.c_void_p),
                ("mep_ic", C.c_void_p), ("mep_lc", C.c_void_p), ("mep_cs", C.c_void_p),
                ("kubo_mep_ic", C.c_void_p), ("kubo_mep_lc", C.c_void_p),
                ("kubo_mep_cs", C.c_void_p), ("n_k", C.c_int64),
                ("velo_ahc", C.c_void_p), ("kubo_ohc", C.c_void_p)]


def _find_zheevd():
    """Return (lib handle, function address) of a LAPACK zheevd."""
    cands = []
    try:
        import scipy
        d = os.path.dirname(scipy.__file__)
        cands += glob.glob(os.path.join(d, "..", "scipy.libs", "*openblas*.so*"))
        cands += glob.glob(os.path.join(d, ".dylibs", "*openblas*"))
    except ImportError:
        pass
    cands += ["liblapack.so.3", "liblapack.so", "libopenblas.so.0"]
    for path in cands:
        try:
            lib = C.CDLL(path)
        except OSError:
            continue
        for sym in ("scipy_zheevd_", "zheevd_"):
            try:
                fn = getattr(lib, sym)
                return lib, C.cast(fn, C.c_void_p).value
            except AttributeError:
                continue
    raise RuntimeError("no LAPACK zheevd found for the C oracle")


_LIB = None
_LAPACK = None


def lib():
    global _LIB, _LAPACK
    if _LIB is None:
        build()
        _LIB = C.CDLL(LIB)
        _LAPACK, addr = _find_zheevd()
        _LIB.oracle_set_zheevd(C.c_void_p(addr))
        _LIB.oracle_run.restype = C.c_int
        _LIB.oracle_run.argtypes = [C.POINTER(_Model), C.POINTER(_Job), C.c_int64, C.c_int64,
                                    C.c_int64, C.POINTER(_Out), C.c_int]
        _LIB.oracle_run_kserial.restype = C.c_int
        _LIB.oracle_run_kserial.argtypes = _LIB.oracle_run.argtypes
        _LIB.oracle_interp_k.restype = C.c_int
    return _LIB


def _fortran_model(model: dict):
    """Convert the numpy-oracle model dict (C-order arrays) to Fortran layouts."""
    H = np.asarray(model["H"], np.complex128)                        # (nR,N,N)
    nR, N, _ = H.shape
    keep = {}
    keep["R"] = np.ascontiguousarray(np.asarray(model["R_frac"], np.float64))        # (nR,3) == (3,nR) F
    keep["H"] = np.ascontiguousarray(H.transpose(0, 2, 1))          # mem order n fastest, then m, then R
    r = model.get("r")
    keep["r"] = None if r is None else np.ascontiguousarray(np.asarray(r, np.complex128).transpose(0, 3, 2, 1))
    tau = model.get("wf_centers")
    keep["tau"] = None if tau is None else np.ascontiguousarray(np.asarray(tau, np.float64))  # (N,3) == (3,N) F
    m = _Model()
    m.n_wf, m.n_R = N, nR
    m.R_frac = keep["R"].ctypes.data
    m.H = keep["H"].ctypes.data
    m.r = 0 if keep["r"] is None else keep["r"].ctypes.data
    m.wf_centers = 0 if keep["tau"] is None else keep["tau"].ctypes.data
    a = np.asarray(model["a_latt"], np.float64)
    for j in range(3):
        for i in range(3):
            m.a_latt[i + 3 * j] = a[i, j]
    m.do_gauge_trafo = int(bool(model.get("do_gauge_trafo", True)))
    m.use_cart_velo = int(bool(model.get("use_cart_velo", False)))
    m.semantics = 0 if model.get("semantics", "ref") == "ref" else 1
    m.kubo_tol = float(model.get("kubo_tol", 1e-5))
    return m, keep


def run(model: dict, job: dict, k_begin: int = 0, k_count=None, k_stride: int = 1, nthreads: int = 0,
        kserial: bool = False) -> dict:
    """Same contract as ref_numpy.run, over k = k_begin + s*k_stride.

    ``kserial=False``: threads share the k-points (OpenMP over k).
    ``kserial=True``: the reference's own structure -- a serial k-loop with the
    Fourier sum of each k split over the threads by R (oracle_run_kserial)."""
    L = lib()
    m, keep = _fortran_model(model)
    mp = [int(x) for x in job["mp_grid"]]
    nk_tot = mp[0] * mp[1] * mp[2]
    if k_count is None:
        k_count = (nk_tot - k_begin + k_stride - 1) // k_stride
    ef = np.ascontiguousarray(np.asarray(job["ef_lst"], np.float64))
    nE = ef.size
    nv = int(job["valence_bands"])
    j = _Job()
    for i in range(3):
        j.mp_grid[i] = mp[i]
    j.n_eF, j.ef_lst, j.T_kelvin, j.valence_bands = nE, ef.ctypes.data, float(job.get("T_kelvin", 0.0)), nv
    j.do_ahc = int(bool(job.get("do_ahc", True)))
    j.do_mep = int(bool(job.get("do_mep", True)))
    j.do_kubo = int(bool(job.get("do_kubo", True)))
    res = {"Ne_sum": np.zeros(nE), "ahc": np.zeros((3, 3, nE), order="F"),
           "mep_ic": np.zeros((3, 3, nv), order="F"), "mep_lc": np.zeros((3, 3, nv), order="F"),
           "mep_cs": np.zeros((3, 3, nv), order="F"),
           "kubo_mep_ic": np.zeros((3, 3, nE), order="F"), "kubo_mep_lc": np.zeros((3, 3, nE), order="F"),
           "kubo_mep_cs": np.zeros((3, 3, nE), order="F")}
    hw = job.get("hw_lst")
    hw = None if hw is None else np.ascontiguousarray(np.asarray(hw, np.float64))
    omega = j.do_ahc and hw is not None and hw.size > 0
    if omega:
        j.n_hw, j.hw_lst, j.eta_smr = hw.size, hw.ctypes.data, float(job.get("eta_smr", 0.0))
        res["velo_ahc"] = np.zeros((3, 3, hw.size, nE), np.complex128, order="F")
        res["kubo_ohc"] = np.zeros((3, 3, hw.size, nE), np.complex128, order="F")
    o = _Out()
    for key in res:
        setattr(o, key, res[key].ctypes.data)
    o.n_k = 0
    fn = L.oracle_run_kserial if kserial else L.oracle_run
    rc = fn(C.byref(m), C.byref(j), int(k_begin), int(k_count), int(k_stride), C.byref(o), int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle_run failed with status {rc}")
    res["n_k"] = int(o.n_k)
    del keep
    return res


def interp_k(model: dict, kpt):
    """E (N,), V (3,N,N), A (3,N,N) | None, Om (3,3,N,N) | None for one k (C-order axes)."""
    L = lib()
    m, keep = _fortran_model(model)
    N = m.n_wf
    k = np.ascontiguousarray(np.asarray(kpt, np.float64))
    E = np.zeros(N)
    V = np.zeros((3, N, N), np.complex128, order="F")
    A = np.zeros((3, N, N), np.complex128, order="F")
    Om = np.zeros((3, 3, N, N), np.complex128, order="F")
    rc = L.oracle_interp_k(C.byref(m), C.c_void_p(k.ctypes.data), C.c_void_p(E.ctypes.data),
                           C.c_void_p(V.ctypes.data), C.c_void_p(A.ctypes.data), C.c_void_p(Om.ctypes.data))
    if rc != 0:
        raise RuntimeError(f"oracle_interp_k failed with status {rc}")
    has_r = model.get("r") is not None
    return E, V, (A if has_r else None), (Om if has_r else None)
