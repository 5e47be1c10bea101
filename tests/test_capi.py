"""CPU checks of the C ABI boundary: the library builds, loads, exports every
function include/*.h declares, its ctypes mirror has mepi.h's struct
layouts, and argument validation answers before any device work."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from mepinterp_gb300 import api, build
from mepinterp_gb300.generator import random_tb_model

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mepi.h")


@pytest.fixture(scope="module")
def lib():
    build.build()
    return api.load_library()


def header_functions():
    inc = os.path.join(ROOT, "include")
    txt = "".join(open(os.path.join(inc, h)).read() for h in sorted(os.listdir(inc)) if h.endswith(".h"))
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(mepi_\w+)\s*\(", txt, flags=re.M)))


def test_exports_every_declared_symbol(lib):
    names = header_functions()
    assert {"mepi_create", "mepi_run", "mepi_destroy", "mepi_strerror", "mepi_interp_k", "mepi_run_batch",
            "mepi_autotune", "mepi_set_mem_limit", "mepi_mlp_create", "mepi_mlp_train"} <= set(names)
    for n in names:
        assert hasattr(lib, n), n


def test_struct_layouts_match_header(tmp_path):
    """sizeof/offsetof from a C compile of mepi.h equal the ctypes mirror's."""
    fields = {"mepi_model": api.MepiModel, "mepi_job": api.MepiJob, "mepi_acc": api.MepiAcc,
              "mepi_timing": api.MepiTiming, "mepi_tuning": api.MepiTuning}
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "mepi.h"', "int main(void){"]
    for cname, cls in fields.items():
        src.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            src.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    src.append("return 0;}")
    c = tmp_path / "probe.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)])
    out = dict(line.split() for line in subprocess.check_output([str(exe)]).decode().splitlines())
    for cname, cls in fields.items():
        assert int(out[cname]) == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(out[f"{cname}.{f}"]) == getattr(cls, f).offset, (cname, f)


def test_strerror_and_version(lib):
    for s in range(7):
        assert lib.mepi_strerror(s)
    assert b"sm_103a" in lib.mepi_version()


def _create(lib, model, mutate=None):
    bufs = api.fortran_model_arrays(model)
    m = api.make_mepi_model(model, bufs)
    if mutate:
        mutate(m, bufs)
    h = C.c_void_p()
    rc = lib.mepi_create(C.byref(h), C.byref(m))
    if rc == 0:
        lib.mepi_destroy(h)
    return rc


def test_create_rejects_bad_arguments(lib):
    model = random_tb_model(n_wf=8, r_max=1, seed=1)
    assert lib.mepi_create(None, None) == api.ERR_ARG

    def zero_n(m, b):
        m.n_wf = 0
    assert _create(lib, model, zero_n) == api.ERR_ARG

    def too_big(m, b):
        m.n_wf = 65
    assert _create(lib, model, too_big) == api.ERR_ARG

    def bad_sem(m, b):
        m.semantics = 7
    assert _create(lib, model, bad_sem) == api.ERR_ARG


def test_create_rejects_nan_and_non_hermitian(lib):
    model = random_tb_model(n_wf=8, r_max=1, seed=1)
    bad = random_tb_model(n_wf=8, r_max=1, seed=1)
    bad.H = bad.H.copy()
    bad.H[3, 1, 2] = np.nan
    assert _create(lib, bad) == api.ERR_NONFINITE
    nh = random_tb_model(n_wf=8, r_max=1, seed=1)
    nh.H = nh.H.copy()
    nh.H[5, 0, 1] += 0.01
    assert _create(lib, nh) == api.ERR_NONHERM
    half = random_tb_model(n_wf=8, r_max=1, seed=1)
    keep = [i for i in range(half.n_R) if tuple(half.R_frac[i]) != (1.0, 0.0, 0.0)]
    half.R_frac, half.H, half.r = half.R_frac[keep], half.H[keep], half.r[keep]
    assert _create(lib, half) == api.ERR_NONHERM
    del model


def test_no_gpu_fails_loudly(lib):
    """Without a CUDA device the library refuses (no CPU fallback exists)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    model = random_tb_model(n_wf=8, r_max=1, seed=1)
    with pytest.raises(api.MepiError) as e:
        api.Context(model)
    assert e.value.status == api.ERR_CUDA


def test_null_contexts_and_bad_counts_are_rejected(lib):
    """The entry points added beside mepi_run answer NULL contexts and bad
    counts with MEPI_ERR_ARG before any device work."""
    P = C.c_void_p
    lib.mepi_trim.argtypes = [P]
    lib.mepi_set_mem_limit.argtypes = [P, C.c_uint64]
    lib.mepi_run_batch.argtypes = [C.c_int32, P, P, P, P]
    assert lib.mepi_trim(None) == api.ERR_ARG
    assert lib.mepi_set_mem_limit(None, 1 << 20) == api.ERR_ARG
    assert lib.mepi_run_batch(-1, None, None, None, None) == api.ERR_ARG
    assert lib.mepi_run_batch(0, None, None, None, None) == api.OK
    assert lib.mepi_run_batch(2, None, None, None, None) == api.ERR_ARG


def test_bandsum_noalloc_checks_arguments_before_device_work(lib):
    """mepi_bandsum_noalloc answers bad arguments on the host, before any CUDA
    call: a Fermi-energy count whose 32-bit slice size would wrap
    (37 * 116080198 = 30 mod 2^32) and any count beyond the fixed scratch
    array give MEPI_ERR_SCRATCH; an unsupported output bit, a non-finite
    temperature and a negative kuboTol give MEPI_ERR_ARG.  The device pointers
    are never dereferenced on these paths."""
    f = lib.mepi_bandsum_noalloc
    f.argtypes = [C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_double,
                  C.c_int32, C.c_uint32, C.c_double, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    fake = C.c_void_p(0x1000)   # stands in for device buffers; never touched

    def call(n_eF=1, T=0.0, nval=4, outputs=7, tol=1e-5):
        return f(8, 1, fake, fake, None, n_eF, fake, T, nval, outputs, tol, fake, None)

    err_scratch = 7
    assert 37 * 116080198 % (1 << 32) == 30
    assert call(n_eF=116080198) == err_scratch
    assert call(n_eF=(1 << 31) - 1) == err_scratch
    assert call(n_eF=91, nval=4) == err_scratch      # 37*91 + 27*4 = 3475 > 3449
    assert call(outputs=8) == api.ERR_ARG            # optical Hall: not offered here
    assert call(outputs=1 << 31) == api.ERR_ARG
    assert call(T=float("inf")) == api.ERR_ARG
    assert call(T=float("nan")) == api.ERR_ARG
    assert call(tol=-1.0) == api.ERR_ARG
    assert call(n_eF=0) == api.ERR_ARG


def test_mlp_create_checks_shape_then_device(lib):
    """mepi_mlp_create rejects bad shapes (n_in 1..64, width 128, depth 1..8)
    with MEPI_ERR_ARG and, without a CUDA device, valid ones with
    MEPI_ERR_CUDA: the network has no CPU fallback."""
    import torch
    f = lib.mepi_mlp_create
    f.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.c_int32, C.c_uint64]
    h = C.c_void_p()
    for n_in, width, depth in ((0, 128, 4), (65, 128, 4), (31, 64, 4), (31, 128, 0), (31, 128, 9)):
        assert f(C.byref(h), n_in, width, depth, 0) == api.ERR_ARG
    assert f(None, 31, 128, 4, 0) == api.ERR_ARG
    if not torch.cuda.is_available():
        assert f(C.byref(h), 31, 128, 4, 0) == api.ERR_CUDA


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "mepi.h"
/* A plain C caller of the k-loop: one-band-pair toy model, a 2^3 mesh. */
int main(void) {
    const double R[3 * 3] = {0, 0, 0, 1, 0, 0, -1, 0, 0};
    double H[2 * 2 * 2 * 3];   /* complex H(2,2,3), column-major */
    memset(H, 0, sizeof H);
    H[0] = -0.1; H[6] = 0.1;                  /* R = 0: diag(-0.1, 0.1) */
    H[8 + 2] = 0.05; H[16 + 4] = 0.05;        /* R = +x: H(2,1); R = -x: H(1,2) = conj */
    mepi_model m;
    memset(&m, 0, sizeof m);
    m.n_wf = 2; m.n_R = 3; m.R_frac = R; m.H = H;
    m.a_latt[0] = m.a_latt[4] = m.a_latt[8] = 5.0;
    m.do_gauge_trafo = 1; m.kubo_tol = 1e-5;
    mepi_ctx *ctx = NULL;
    int rc = mepi_create(&ctx, &m);
    if (rc == MEPI_OK) {
        const double ef = 0.0;
        double ahc[9], ne;
        mepi_job j;
        memset(&j, 0, sizeof j);
        j.mp_grid[0] = j.mp_grid[1] = j.mp_grid[2] = 2; j.k_stride = 1; j.k_count = -1;
        j.n_eF = 1; j.ef_lst = &ef; j.valence_bands = 1; j.outputs = MEPI_OUT_AHC; j.degen_gap = -1;
        mepi_acc a;
        memset(&a, 0, sizeof a);
        a.ahc = ahc; a.Ne_sum = &ne;
        rc = mepi_run(ctx, &j, &a);
        if (rc == MEPI_OK) printf("n_k %lld Ne %.6f\n", (long long)a.n_k_done, ne);
        mepi_destroy(ctx);
    }
    printf("status %d %s\n", rc, mepi_strerror(rc));
    return 0;
}
"""


def test_plain_c_caller_links_and_runs(lib, tmp_path):
    """The C ABI used from plain C (as a Fortran shim or a C++ driver would):
    the program compiles against include/mepi.h, links libmepi_gb300.so and
    runs; without a GPU mepi_create answers MEPI_ERR_CUDA, with one the 2^3
    mesh of the toy model is summed (8 k-points, one electron each)."""
    import torch
    c = tmp_path / "caller.c"
    c.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(build.LIB)
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-L", libdir, "-lmepi_gb300",
                           f"-Wl,-rpath,{libdir}", "-o", str(exe)])
    out = subprocess.check_output([str(exe)]).decode()
    if torch.cuda.is_available():
        assert "status 0" in out and "n_k 8 Ne 8.000000" in out, out
    else:
        assert f"status {api.ERR_CUDA}" in out, out
