"""GPU test of mepi_bandsum_noalloc, the entry point that allocates nothing.

It exists for callers that cannot allocate device memory when they want the
band sums (all device memory handed to their own pool at start-up, a fixed
device-memory budget, or no room for cudaMalloc's latency and implicit
synchronisation).  The test holds the inputs and outputs in caller-owned
device buffers, calls the entry point through the C ABI twice in a row, and
checks both results against the oracle's sums over the same k-points (the
energies, velocities and Chern-Simons values come from the library's FP64
per-k interpolation, which the parity tests pin to the oracle), within the
1e-8 relative tolerance of the FP64 parity tests.  The cases cover every
output family, a single family (the others must come back as zeros), a NULL
Chern-Simons input, and more k-points than the variant's 152 CTAs so that each
CTA walks several k-points.  It also checks that a problem larger than the
fixed scratch array is rejected.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from mepinterp_gb300 import api
from mepinterp_gb300.generator import random_tb_model
from oracle import ref_numpy as O

pytestmark = pytest.mark.gpu

SUM_TOL = 1e-8
ERR_SCRATCH = 7
OUT_AHC, OUT_MEP, OUT_KUBO = 1, 2, 4


def _bind(lib):
    f = lib.mepi_bandsum_noalloc
    f.argtypes = [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_double,
                  C.c_int32, C.c_uint32, C.c_double, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _csv(A, Om):
    """0.5 Re(sum_c conj(A_c(n,n)) om_c(n)), om_c = sum_ab eps_abc Om_ab."""
    om = np.stack([Om[:, 1, 2] - Om[:, 2, 1], Om[:, 2, 0] - Om[:, 0, 2], Om[:, 0, 1] - Om[:, 1, 0]], axis=1)
    return 0.5 * np.einsum("kcn,kcn->kn", np.conj(A), om).real


def _rel(a, b):
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / scale) if scale > 0 else float(np.abs(a).max())


def _unpack(s, nE, nval):
    return {"Ne_sum": s[:nE], "ahc": s[nE:10 * nE], "kubo_mep_ic": s[10 * nE:19 * nE],
            "kubo_mep_lc": s[19 * nE:28 * nE], "kubo_mep_cs": s[28 * nE:37 * nE],
            "mep_ic": s[37 * nE:37 * nE + 9 * nval], "mep_lc": s[37 * nE + 9 * nval:37 * nE + 18 * nval],
            "mep_cs": s[37 * nE + 18 * nval:]}


FAMILY = {"ahc": OUT_AHC, "mep_ic": OUT_MEP, "mep_lc": OUT_MEP, "mep_cs": OUT_MEP,
          "kubo_mep_ic": OUT_KUBO, "kubo_mep_lc": OUT_KUBO, "kubo_mep_cs": OUT_KUBO}


@pytest.mark.parametrize("mesh,outputs,with_csv", [((4, 4, 4), 7, True), ((8, 8, 8), 7, True),
                                                   ((8, 8, 8), OUT_AHC, True), ((5, 5, 5), 7, False)])
def test_noalloc_matches_oracle(gpu_lib, mesh, outputs, with_csv):
    import torch
    fn = _bind(gpu_lib)
    model = random_tb_model(n_wf=8, r_max=1, seed=1)
    ef = np.array([-0.02, 0.0, 0.01])
    nval, N = 4, 8
    nk = int(np.prod(mesh))
    job = dict(mp_grid=mesh, ef_lst=ef, T_kelvin=300.0, valence_bands=nval)
    kpts = O.rel_kpts(mesh, np.arange(nk))
    with api.Context(model) as ctx:
        E, V, A, Om = ctx.get_wann_interp(kpts, precision=api.PREC_FP64)
    ref = O.run(model.as_dict(), job, batch=128)
    dev = torch.device("cuda:0")
    d_E = torch.from_numpy(np.ascontiguousarray(E)).to(dev)
    d_V = torch.from_numpy(np.ascontiguousarray(V).view(np.float64)).to(dev)   # [k][a][n][m] (re, im)
    d_csv = torch.from_numpy(np.ascontiguousarray(_csv(A, Om))).to(dev) if with_csv else None
    d_ef = torch.from_numpy(ef).to(dev)
    size = 37 * ef.size + 27 * nval
    stream = torch.cuda.current_stream(dev).cuda_stream
    for _call in range(2):
        d_sums = torch.full((size,), np.nan, dtype=torch.float64, device=dev)
        rc = fn(N, nk, d_E.data_ptr(), d_V.data_ptr(), d_csv.data_ptr() if with_csv else None, ef.size,
                d_ef.data_ptr(), 300.0, nval, outputs, 1e-5, d_sums.data_ptr(), C.c_void_p(stream))
        assert rc == 0, gpu_lib.mepi_strerror(rc)
        torch.cuda.synchronize()
        got = _unpack(d_sums.cpu().numpy(), ef.size, nval)
        assert _rel(got["Ne_sum"], ref["Ne_sum"]) < SUM_TOL
        for k, fam in FAMILY.items():
            r = np.asarray(ref[k]).ravel(order="F")
            if outputs & fam and (with_csv or not k.endswith("_cs")):
                assert _rel(got[k], r) < SUM_TOL, (k, _rel(got[k], r))
            else:   # family not asked for, or no Chern-Simons input: zeros
                assert np.all(got[k] == 0.0), k


def test_noalloc_rejects_oversized_problem(gpu_lib):
    import torch
    fn = _bind(gpu_lib)
    dev = torch.device("cuda:0")
    d = torch.zeros(1024, dtype=torch.float64, device=dev)
    # 37 * 100 + 27 * 4 > 3449: beyond the fixed scratch array
    rc = fn(8, 1, d.data_ptr(), d.data_ptr(), None, 100, d.data_ptr(), 0.0, 4, 7, 1e-5, d.data_ptr(), None)
    assert rc == ERR_SCRATCH
