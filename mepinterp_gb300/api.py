"""Python front end of the C ABI in include/mepi.h (libmepi_gb300.so).

This mirrors the reference's call surface for the hot path:

* :class:`Context` holds one uploaded tight-binding basis (``mepi_create``), as
  ``read_tb_basis`` leaves it for ``core_worker`` (src/core.f90:144).
* :meth:`Context.core_worker_loc` runs the k-loop body of one rank
  (src/core.f90:165-270) and returns the reference's unnormalised ``*_loc``
  sums (Ne_loc_sum, kubo_ahc_loc, mep_bands_*_loc, kubo_mep_*_loc).
* :meth:`Context.get_wann_interp` returns, per k-point, what get_wann_interp
  (src/wann_interp.f90:56-108) produces that the band sums consume: en_k, V_ka
  and the band diagonals of A_ka and Om_kab.

The library is the only compute path: there is no CPU fallback, and every call
raises :class:`MepiError` when the library cannot be loaded or the GPU call
fails.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from .generator import TBModel

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmepi_gb300.so")

OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_EIG, ERR_NONHERM, ERR_NONFINITE = range(7)
SEM_REF, SEM_PAPER = 0, 1
OUT_AHC, OUT_MEP_NIU, OUT_KUBO_MEP, OUT_OPT_HALL = 1, 2, 4, 8
PREC_FP64, PREC_MIXED = 0, 1


class MepiError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"mepi status {status}: {msg}")
        self.status = status


class MepiModel(C.Structure):
    _fields_ = [("n_wf", C.c_int32), ("n_R", C.c_int32),
                ("R_frac", C.c_void_p), ("H", C.c_void_p), ("r", C.c_void_p),
                ("wf_centers", C.c_void_p), ("a_latt", C.c_double * 9),
                ("do_gauge_trafo", C.c_int32), ("use_cart_velo", C.c_int32),
                ("semantics", C.c_int32), ("kubo_tol", C.c_double)]


class MepiJob(C.Structure):
    _fields_ = [("mp_grid", C.c_int32 * 3), ("k_begin", C.c_int64), ("k_stride", C.c_int64),
                ("k_count", C.c_int64), ("n_eF", C.c_int32), ("ef_lst", C.c_void_p),
                ("T_kelvin", C.c_double), ("valence_bands", C.c_int32), ("outputs", C.c_uint32),
                ("precision", C.c_int32), ("chunk_k", C.c_int64), ("degen_gap", C.c_double),
                ("n_hw", C.c_int32), ("hw_lst", C.c_void_p), ("eta_smr", C.c_double), ("k_list", C.c_void_p)]


class MepiAcc(C.Structure):
    _fields_ = [("Ne_sum", C.c_void_p), ("ahc", C.c_void_p),
                ("mep_ic", C.c_void_p), ("mep_lc", C.c_void_p), ("mep_cs", C.c_void_p),
                ("kubo_mep_ic", C.c_void_p), ("kubo_mep_lc", C.c_void_p), ("kubo_mep_cs", C.c_void_p),
                ("n_k_done", C.c_int64), ("n_k_fp64", C.c_int64), ("eig_max_sweeps", C.c_int32),
                ("velo_ahc", C.c_void_p), ("kubo_ohc", C.c_void_p), ("perk", C.c_void_p)]


STAGES = ("ft", "phase", "fth", "eig", "refine", "rot", "gauge", "bandsum", "reduce")


class MepiTiming(C.Structure):
    _fields_ = ([(f"{s}_ms", C.c_double) for s in ("ft", "phase", "fth", "eig", "refine", "rot", "gauge",
                                                   "bandsum", "reduce", "total", "run")]
                + [(f"{s}_launches", C.c_int32) for s in STAGES]
                + [("n_k", C.c_int64), ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64), ("plan_ms", C.c_double)])


_lib: Optional[C.CDLL] = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load libmepi_gb300.so; raises MepiError if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise MepiError(ERR_CUDA, f"{path} is missing; build it with `python -m mepinterp_gb300.build`")
    lib = C.CDLL(path)
    P = C.c_void_p
    lib.mepi_create.argtypes = [C.POINTER(P), C.POINTER(MepiModel)]
    lib.mepi_create.restype = C.c_int
    lib.mepi_run.argtypes = [P, C.POINTER(MepiJob), C.POINTER(MepiAcc)]
    lib.mepi_run.restype = C.c_int
    lib.mepi_interp_k.argtypes = [P, C.c_int32, C.c_int64, P, P, P, P, P]
    lib.mepi_interp_k.restype = C.c_int
    lib.mepi_get_timing.argtypes = [P, C.POINTER(MepiTiming)]
    lib.mepi_get_timing.restype = C.c_int
    lib.mepi_destroy.argtypes = [P]
    lib.mepi_destroy.restype = C.c_int
    lib.mepi_autotune.argtypes = [P, C.POINTER(MepiJob), C.c_int64, C.POINTER(MepiTuning)]
    lib.mepi_autotune.restype = C.c_int
    lib.mepi_set_tuning.argtypes = [P, C.POINTER(MepiTuning)]
    lib.mepi_set_tuning.restype = C.c_int
    lib.mepi_set_mem_limit.argtypes = [P, C.c_uint64]
    lib.mepi_set_mem_limit.restype = C.c_int
    lib.mepi_trim.argtypes = [P]
    lib.mepi_trim.restype = C.c_int
    lib.mepi_get_tuning.argtypes = [P, C.POINTER(MepiTuning)]
    lib.mepi_get_tuning.restype = C.c_int
    lib.mepi_run_batch.argtypes = [C.c_int32, C.POINTER(P), C.POINTER(MepiJob), C.POINTER(MepiAcc),
                                   C.POINTER(C.c_double)]
    lib.mepi_run_batch.restype = C.c_int
    lib.mepi_strerror.argtypes = [C.c_int]
    lib.mepi_strerror.restype = C.c_char_p
    lib.mepi_version.restype = C.c_char_p
    _lib = lib
    return lib


def _check(status: int):
    if status != OK:
        msg = load_library().mepi_strerror(status).decode()
        raise MepiError(status, msg)


def fortran_model_arrays(model: TBModel) -> dict:
    """Fortran-layout (column-major) host buffers the C ABI takes."""
    H = np.asarray(model.H, np.complex128)
    out = {
        # R_frac(3,nR): memory order component fastest == C-order (nR,3)
        "R": np.ascontiguousarray(np.asarray(model.R_frac, np.float64)),
        # H(N,N,nR): n fastest, then m, then R == C-order [R][m][n]
        "H": np.ascontiguousarray(H.transpose(0, 2, 1)),
        "r": None, "tau": None,
    }
    if model.r is not None:
        # r(3,N,N,nR): a fastest, then n, m, R == C-order [R][m][n][a]
        out["r"] = np.ascontiguousarray(np.asarray(model.r, np.complex128).transpose(0, 3, 2, 1))
    if model.wf_centers is not None:
        out["tau"] = np.ascontiguousarray(np.asarray(model.wf_centers, np.float64))
    return out


def make_mepi_model(model: TBModel, bufs: dict) -> MepiModel:
    m = MepiModel()
    m.n_wf = model.n_wf
    m.n_R = model.n_R
    m.R_frac = bufs["R"].ctypes.data
    m.H = bufs["H"].ctypes.data
    m.r = bufs["r"].ctypes.data if bufs["r"] is not None else None
    m.wf_centers = bufs["tau"].ctypes.data if bufs["tau"] is not None else None
    a = np.asarray(model.a_latt, np.float64)
    for j in range(3):
        for i in range(3):
            m.a_latt[i + 3 * j] = a[i, j]
    m.do_gauge_trafo = int(bool(model.do_gauge_trafo))
    m.use_cart_velo = int(bool(model.use_cart_velo))
    m.semantics = SEM_REF if model.semantics == "ref" else SEM_PAPER
    m.kubo_tol = float(model.kubo_tol)
    return m


class Context:
    """One tight-binding basis resident on the GPU (mepi_create / mepi_destroy)."""

    def __init__(self, model: TBModel):
        self.lib = load_library()
        self.model = model
        bufs = fortran_model_arrays(model)
        m = make_mepi_model(model, bufs)
        h = C.c_void_p()
        _check(self.lib.mepi_create(C.byref(h), C.byref(m)))
        self._h = h
        self.n_wf = model.n_wf

    def close(self):
        if getattr(self, "_h", None):
            self.lib.mepi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------------
    def core_worker_loc(self, job: dict, precision: int = PREC_FP64, k_begin: int = 0, k_stride: int = 1,
                        k_count: int = -1, chunk_k: int = 0, degen_gap: float = -1.0, k_list=None,
                        perk: bool = False) -> dict:
        """k-loop body of src/core.f90:165-270 for k = k_begin + s*k_stride
        (or for the mesh indices ``k_list``).

        ``job`` keys: mp_grid, ef_lst (Hartree), T_kelvin, valence_bands and
        optionally do_ahc / do_mep / do_kubo (default True), and hw_lst
        (Hartree) with eta_smr for the optical Hall tensors velo_ahc and
        kubo_ohc (3,3,n_hw,n_eF) that the reference computes with do_ahc.
        Returns the unnormalised local sums with the reference's shapes
        (Fortran order); with ``perk`` also "perk" (n_k, 4): per k-point the
        (y,z), (z,x), (x,y) entries of its AHC term at ef_lst[0] and the band
        gap across ef_lst[0].
        """
        call = _JobCall(job, precision, k_begin, k_stride, k_count, chunk_k, degen_gap, k_list, perk)
        _check(self.lib.mepi_run(self._h, C.byref(call.j), C.byref(call.acc)))
        return call.result()

    def autotune(self, job: dict, precision: int = PREC_MIXED, sample_k: int = 0) -> dict:
        """mepi_autotune: time the candidate launch shapes on the first sample_k
        k-points of the job and keep the fastest for this context (and for
        later contexts of the same kind in this process)."""
        call = _JobCall(job, precision)
        t = MepiTuning()
        _check(self.lib.mepi_autotune(self._h, C.byref(call.j), int(sample_k), C.byref(t)))
        return {f: getattr(t, f) for f, _ in MepiTuning._fields_}

    def get_tuning(self) -> dict:
        t = MepiTuning()
        _check(self.lib.mepi_get_tuning(self._h, C.byref(t)))
        return {f: getattr(t, f) for f, _ in MepiTuning._fields_}

    def set_tuning(self, jacobi_threads: int = 0, jacobi_kblock: int = 0, chunk_k: int = 0) -> None:
        t = MepiTuning(int(jacobi_threads), int(jacobi_kblock), int(chunk_k), 0.0)
        _check(self.lib.mepi_set_tuning(self._h, C.byref(t)))

    def set_mem_limit(self, nbytes: int) -> None:
        """Device-memory limit for the separable slabs and chunk buffers (0 =
        the defaults); a large mesh under a small limit builds its slabs one
        qx range at a time.  Results do not depend on it."""
        _check(self.lib.mepi_set_mem_limit(self._h, int(nbytes)))

    def trim(self) -> None:
        """mepi_trim: free the cached slabs and chunk buffers (rebuilt on the next run)."""
        _check(self.lib.mepi_trim(self._h))

    def get_wann_interp(self, kpts, precision: int = PREC_FP64):
        """en_k (nk,N), V (nk,3,N,N), A_diag (nk,3,N), Om_diag (nk,3,3,N) in C order."""
        k = np.ascontiguousarray(np.atleast_2d(np.asarray(kpts, np.float64)))
        nk, N = k.shape[0], self.n_wf
        E = np.zeros((nk, N))
        V = np.zeros((nk, N, N, 3), np.complex128)       # Fortran (3,N,N,nk) memory order
        A = np.zeros((nk, N, 3), np.complex128)
        Om = np.zeros((nk, N, 3, 3), np.complex128)
        _check(self.lib.mepi_interp_k(self._h, int(precision), nk, k.ctypes.data, E.ctypes.data, V.ctypes.data,
                                      A.ctypes.data, Om.ctypes.data))
        # Fortran V_ka(a,n,m,k): memory a fastest, then n, then m -> C array [k][m][n][a]
        V = V.transpose(0, 3, 2, 1)                      # -> [k][a][n][m]
        A = A.transpose(0, 2, 1)                         # [k][n][c] -> [k][c][n]
        Om = Om.transpose(0, 3, 2, 1)                    # [k][n][b][a] -> [k][a][b][n]
        return E, V, A, Om

    def timing(self) -> dict:
        t = MepiTiming()
        _check(self.lib.mepi_get_timing(self._h, C.byref(t)))
        return {f: getattr(t, f) for f, _ in MepiTiming._fields_}


class MepiTuning(C.Structure):
    _fields_ = [("jacobi_threads", C.c_int32), ("jacobi_kblock", C.c_int32), ("chunk_k", C.c_int64),
                ("k_per_s", C.c_double)]


class _JobCall:
    """A mepi_job and its mepi_acc with the result arrays they point to."""

    def __init__(self, job: dict, precision: int = PREC_FP64, k_begin: int = 0, k_stride: int = 1,
                 k_count: int = -1, chunk_k: int = 0, degen_gap: float = -1.0, k_list=None, perk: bool = False):
        self.ef = np.ascontiguousarray(np.atleast_1d(np.asarray(job["ef_lst"], np.float64)))
        nE = self.ef.size
        nv = int(job["valence_bands"])
        j = MepiJob()
        for i in range(3):
            j.mp_grid[i] = int(job["mp_grid"][i])
        j.k_begin, j.k_stride, j.k_count = int(k_begin), int(k_stride), int(k_count)
        self.k_list = None
        n_tot = int(np.prod([int(x) for x in job["mp_grid"]]))
        if k_list is not None:
            self.k_list = np.ascontiguousarray(np.asarray(k_list, np.int64).ravel())
            j.k_list, j.k_count, j.k_begin, j.k_stride = self.k_list.ctypes.data, self.k_list.size, 0, 1
            n_k = self.k_list.size
        else:
            owned = max(0, -(-(n_tot - int(k_begin)) // int(k_stride))) if int(k_stride) > 0 else 0
            n_k = owned if int(k_count) < 0 else min(int(k_count), owned)
        j.n_eF, j.ef_lst = nE, self.ef.ctypes.data
        j.T_kelvin = float(job.get("T_kelvin", 0.0))
        j.valence_bands = nv
        outs = 0
        if job.get("do_ahc", True):
            outs |= OUT_AHC
        if job.get("do_mep", True):
            outs |= OUT_MEP_NIU
        if job.get("do_kubo", True):
            outs |= OUT_KUBO_MEP
        hw = job.get("hw_lst")
        self.hw = None if hw is None else np.ascontiguousarray(np.atleast_1d(np.asarray(hw, np.float64)))
        if (outs & OUT_AHC) and self.hw is not None and self.hw.size:
            outs |= OUT_OPT_HALL
            j.n_hw, j.hw_lst, j.eta_smr = self.hw.size, self.hw.ctypes.data, float(job.get("eta_smr", 0.0))
        j.outputs = outs
        j.precision = int(precision)
        j.chunk_k = int(chunk_k)
        j.degen_gap = float(degen_gap)
        self.j = j
        self.res = {"Ne_sum": np.zeros(nE), "ahc": np.zeros((3, 3, nE), order="F"),
                    "mep_ic": np.zeros((3, 3, nv), order="F"), "mep_lc": np.zeros((3, 3, nv), order="F"),
                    "mep_cs": np.zeros((3, 3, nv), order="F"),
                    "kubo_mep_ic": np.zeros((3, 3, nE), order="F"), "kubo_mep_lc": np.zeros((3, 3, nE), order="F"),
                    "kubo_mep_cs": np.zeros((3, 3, nE), order="F")}
        if outs & OUT_OPT_HALL:
            self.res["velo_ahc"] = np.zeros((3, 3, self.hw.size, nE), np.complex128, order="F")
            self.res["kubo_ohc"] = np.zeros((3, 3, self.hw.size, nE), np.complex128, order="F")
        if perk:
            self.res["perk"] = np.zeros((n_k, 4))
        self.acc = MepiAcc()
        for key, arr in self.res.items():
            setattr(self.acc, key, arr.ctypes.data if arr.size else None)

    def result(self) -> dict:
        res = dict(self.res)
        res["n_k"] = int(self.acc.n_k_done)
        res["n_k_fp64"] = int(self.acc.n_k_fp64)
        res["eig_max_sweeps"] = int(self.acc.eig_max_sweeps)
        return res


def run_batch(contexts, jobs, precision=PREC_MIXED, perk: bool = False):
    """mepi_run_batch: one (context, job) pair per model, all in one CUDA graph
    launch.  ``precision`` is one value or one per job; with ``perk`` every
    result also holds "perk" (see :meth:`Context.core_worker_loc`).  Returns
    (list of the unnormalised local sums, device time of the graph in ms)."""
    precs = precision if isinstance(precision, (list, tuple)) else [precision] * len(jobs)
    calls = [_JobCall(j, p, perk=perk) for j, p in zip(jobs, precs)]
    n = len(calls)
    lib = contexts[0].lib
    ctxs = (C.c_void_p * n)(*[c._h.value for c in contexts])
    job_arr = (MepiJob * n)(*[c.j for c in calls])
    acc_arr = (MepiAcc * n)(*[c.acc for c in calls])
    ms = C.c_double(0.0)
    _check(lib.mepi_run_batch(n, ctxs, job_arr, acc_arr, C.byref(ms)))
    out = []
    for i, c in enumerate(calls):
        c.acc = acc_arr[i]
        out.append(c.result())
    return out, float(ms.value)


def run(model: TBModel, job: dict, precision: int = PREC_FP64, **kw) -> dict:
    """One-shot: upload the model, run the k-loop, return the *_loc sums."""
    with Context(model) as ctx:
        return ctx.core_worker_loc(job, precision=precision, **kw)
