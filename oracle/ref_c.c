/*
 * CPU oracle (C) for MEPinterp's per-k-point Wannier-interpolation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker and the timed CPU
 * baseline ("port" of the reference loop structure).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The CUDA
 * product never links or calls it.
 *
 * It follows the reference line by line (file:line within cMax347/MEPinterp):
 *   k-loop body ......... src/core.f90:165-270
 *   FT_R_to_k ........... src/wann_interp.f90:151-384 (one sin/cos per (R,n,m))
 *   zheevd_wrapper ...... src/matrix_math.f90:192-226 (LAPACK zheevd, V/U)
 *   rotate_gauge ........ src/wann_interp.f90:502-550
 *   covariant deriv ..... src/wann_interp.f90:565-617
 *   conn/curv trafo ..... src/wann_interp.f90:620-658 (54 zgemm per k)
 *   get_velo ............ src/wann_interp.f90:406-444
 *   fd_stat / N_el ...... src/statistics.f90:41-124
 *   kubo_ahc_tens ....... src/kubo.f90:37-78
 *   velo_ahc_tens,
 *   kubo_ohc_tens ....... src/kubo.f90:86-198
 *   mep_niu_* ........... src/mep_niu.f90:20-159
 *   kubo_mep_* .......... src/kubo_mep.f90:16-149
 * with the same documented positions on D1 (A_bar = U^dag A U), D2
 * (V_nn = Hbar_nn), D3 (alpha = 1, beta = 0) and D4/D5 (replicated in
 * semantics 0 = "ref", A_bar used in semantics 1 = "paper").
 *
 * Arrays use the reference's Fortran (column-major) layout:
 *   R_frac(3,nR), H(N,N,nR) complex, r(3,N,N,nR) complex, tau(3,N),
 *   a_latt(3,3); outputs ahc(3,3,n_eF), mep_*(3,3,n_val), kubo_mep_*(3,3,n_eF).
 * LAPACK zheevd is supplied by the caller as a function pointer (the host
 * LAPACK; scipy's bundled OpenBLAS exports it as scipy_zheevd_).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex zc;

typedef void (*zheevd_fn)(const char *jobz, const char *uplo, const int *n, zc *a,
                          const int *lda, double *w, zc *work, const int *lwork,
                          double *rwork, const int *lrwork, int *iwork,
                          const int *liwork, int *info, size_t, size_t);

typedef struct {
    int32_t n_wf, n_R;
    const double *R_frac;     /* (3,nR) */
    const double *H;          /* (N,N,nR) complex interleaved */
    const double *r;          /* (3,N,N,nR) complex or NULL */
    const double *wf_centers; /* (3,N) or NULL */
    double a_latt[9];         /* (3,3) column-major */
    int32_t do_gauge_trafo, use_cart_velo, semantics;
    double kubo_tol;
} oracle_model;

typedef struct {
    int32_t mp_grid[3];
    int32_t n_eF;
    const double *ef_lst;
    double T_kelvin;
    int32_t valence_bands;
    int32_t do_ahc, do_mep, do_kubo;
    int32_t n_hw;             /* 0: no optical Hall tensors */
    const double *hw_lst;     /* (n_hw) Hartree */
    double eta_smr;           /* smearing: the reference's i_eta_smr = i * eta */
} oracle_job;

typedef struct {
    double *Ne_sum;       /* (n_eF) */
    double *ahc;          /* (3,3,n_eF) */
    double *mep_ic, *mep_lc, *mep_cs;                /* (3,3,n_val) */
    double *kubo_mep_ic, *kubo_mep_lc, *kubo_mep_cs; /* (3,3,n_eF) */
    int64_t n_k;
    double *velo_ahc, *kubo_ohc;  /* (3,3,n_hw,n_eF) complex interleaved, or NULL */
} oracle_out;

static zheevd_fn g_zheevd = 0;
void oracle_set_zheevd(void *fn) { g_zheevd = (zheevd_fn)fn; }

/* src/constants.f90 */
static const double PI_DP = 3.14159265358979323846264338327950288;
#define AU_TO_EV 27.211385
#define KB_EH_K (8.6173303e-5 / AU_TO_EV)
#define MIN_TEMP 1e-2

static int levi(int i, int j, int k) { /* src/matrix_math.f90:125-139 */
    if ((i == 0 && j == 1 && k == 2) || (i == 1 && j == 2 && k == 0) || (i == 2 && j == 0 && k == 1)) return 1;
    if ((i == 0 && j == 2 && k == 1) || (i == 2 && j == 1 && k == 0) || (i == 1 && j == 0 && k == 2)) return -1;
    return 0;
}

/* index helpers: Fortran layouts */
#define IX2(n, m, N) ((n) + (size_t)(N) * (m))
#define IXA(a, n, m, N) ((a) + 3 * ((n) + (size_t)(N) * (m)))
#define IXAB(a, b, n, m, N) ((a) + 3 * ((b) + 3 * ((n) + (size_t)(N) * (m))))

typedef struct {
    int N;
    zc *Hk, *Hka, *Aka, *Omk, *V, *D, *tmp, *tmp2, *Min, *U;
    double *E, *rwork;
    zc *work;
    int *iwork;
    double *fd; /* (n_eF,N) */
} ws_t;

static ws_t ws_alloc(int N, int n_eF) {
    ws_t w;
    size_t NN = (size_t)N * N;
    w.N = N;
    w.Hk = calloc(NN, sizeof(zc));
    w.U = calloc(NN, sizeof(zc));
    w.Hka = calloc(3 * NN, sizeof(zc));
    w.Aka = calloc(3 * NN, sizeof(zc));
    w.Omk = calloc(9 * NN, sizeof(zc));
    w.V = calloc(3 * NN, sizeof(zc));
    w.D = calloc(3 * NN, sizeof(zc));
    w.tmp = calloc(NN, sizeof(zc));
    w.tmp2 = calloc(NN, sizeof(zc));
    w.Min = calloc(NN, sizeof(zc));
    w.E = calloc(N, sizeof(double));
    w.work = calloc(NN + 2 * N, sizeof(zc));
    w.rwork = calloc(2 * NN + 5 * N + 1, sizeof(double));
    w.iwork = calloc(5 * N + 3, sizeof(int));
    w.fd = calloc((size_t)(n_eF > 0 ? n_eF : 1) * N, sizeof(double));
    return w;
}

static void ws_free(ws_t *w) {
    free(w->Hk); free(w->U); free(w->Hka); free(w->Aka); free(w->Omk); free(w->V);
    free(w->D); free(w->tmp); free(w->tmp2); free(w->Min); free(w->E); free(w->work);
    free(w->rwork); free(w->iwork); free(w->fd);
}

/* C = A*B for column-major N x N (zgemm 'N','N' with alpha=1, beta=0; D3) */
static void zmm(int N, const zc *A, const zc *B, zc *C) {
    for (int j = 0; j < N; ++j) {
        for (int i = 0; i < N; ++i) C[IX2(i, j, N)] = 0;
        for (int l = 0; l < N; ++l) {
            zc b = B[IX2(l, j, N)];
            for (int i = 0; i < N; ++i) C[IX2(i, j, N)] += A[IX2(i, l, N)] * b;
        }
    }
}

/* C = A^dag * B */
static void zmm_dagA(int N, const zc *A, const zc *B, zc *C) {
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            zc s = 0;
            for (int l = 0; l < N; ++l) s += conj(A[IX2(l, i, N)]) * B[IX2(l, j, N)];
            C[IX2(i, j, N)] = s;
        }
}

/* copy strided component (a-th of 3 or (a,b)-th of 9) out of / into a plain matrix */
static void get_comp(int N, const zc *X, int stride, int off, zc *M) {
    for (int m = 0; m < N; ++m)
        for (int n = 0; n < N; ++n) M[IX2(n, m, N)] = X[off + (size_t)stride * IX2(n, m, N)];
}
static void put_comp(int N, zc *X, int stride, int off, const zc *M) {
    for (int m = 0; m < N; ++m)
        for (int n = 0; n < N; ++n) X[off + (size_t)stride * IX2(n, m, N)] = M[IX2(n, m, N)];
}

/* ---------------- FT_R_to_k (src/wann_interp.f90:151-384) ---------------- */
static void ft_zero(int N, ws_t *w) {
    const size_t NN = (size_t)N * N;
    memset(w->Hk, 0, NN * sizeof(zc));
    memset(w->Hka, 0, 3 * NN * sizeof(zc));
    memset(w->Aka, 0, 3 * NN * sizeof(zc));
    memset(w->Omk, 0, 9 * NN * sizeof(zc));
}

/* adds the terms of R vectors sc0 <= sc < sc1 into w's Hk, Hka, Aka, Omk */
static void ft_accum(const oracle_model *md, const double kpt[3], ws_t *w, int sc0, int sc1) {
    const int N = md->n_wf;
    const size_t NN = (size_t)N * N;
    const zc *H = (const zc *)md->H;
    const zc *r = (const zc *)md->r;
    const double *a = md->a_latt; /* column-major a(i,j) = a[i+3j] */
    const double two_pi = 2.0 * PI_DP;
    const int use_pos = (r != 0);
    /* kpt_cart = matmul(recip_latt, kpt) (src/k_space.f90:378-396) */
    double kc[3] = {0, 0, 0};
    if (md->use_cart_velo) {
        const double a1[3] = {a[0], a[1], a[2]}, a2[3] = {a[3], a[4], a[5]}, a3[3] = {a[6], a[7], a[8]};
        double c23[3] = {a2[1] * a3[2] - a2[2] * a3[1], a2[2] * a3[0] - a2[0] * a3[2], a2[0] * a3[1] - a2[1] * a3[0]};
        double c31[3] = {a3[1] * a1[2] - a3[2] * a1[1], a3[2] * a1[0] - a3[0] * a1[2], a3[0] * a1[1] - a3[1] * a1[0]};
        double c12[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2], a1[0] * a2[1] - a1[1] * a2[0]};
        double vol = c12[0] * a3[0] + c12[1] * a3[1] + c12[2] * a3[2];
        for (int i = 0; i < 3; ++i)
            kc[i] = (2 * PI_DP * c23[i] / vol) * kpt[0] + (2 * PI_DP * c31[i] / vol) * kpt[1] +
                    (2 * PI_DP * c12[i] / vol) * kpt[2];
    }
    const double *tau = md->wf_centers;
    for (int sc = sc0; sc < sc1; ++sc) {
        const double *R = md->R_frac + 3 * sc;
        for (int m = 0; m < N; ++m)
            for (int n = 0; n < N; ++n) {
                double dR[3];
                for (int i = 0; i < 3; ++i)
                    dR[i] = R[i] + (tau ? (tau[i + 3 * m] - tau[i + 3 * n]) : 0.0);
                double dRc[3];
                if (md->use_cart_velo) {
                    for (int i = 0; i < 3; ++i) dRc[i] = a[i] * dR[0] + a[i + 3] * dR[1] + a[i + 6] * dR[2];
                } else {
                    for (int i = 0; i < 3; ++i) dRc[i] = two_pi * dR[i];
                }
                double ang;
                if (tau && md->use_cart_velo)
                    ang = kc[0] * dRc[0] + kc[1] * dRc[1] + kc[2] * dRc[2];
                else
                    ang = two_pi * (kpt[0] * dR[0] + kpt[1] * dR[1] + kpt[2] * dR[2]);
                zc ph = cos(ang) + I * sin(ang);
                zc h = H[IX2(n, m, N) + NN * sc];
                w->Hk[IX2(n, m, N)] += ph * h;
                for (int i = 0; i < 3; ++i) w->Hka[IXA(i, n, m, N)] += ph * (I * dRc[i]) * h;
                if (use_pos) {
                    /* conn/curv part always uses the internal angle (:306, :348) */
                    double angA = two_pi * (kpt[0] * dR[0] + kpt[1] * dR[1] + kpt[2] * dR[2]);
                    zc phA = cos(angA) + I * sin(angA);
                    for (int i = 0; i < 3; ++i) {
                        zc ri = r[IXA(i, n, m, N) + 3 * NN * sc];
                        w->Aka[IXA(i, n, m, N)] += phA * ri;
                        for (int b = 0; b < 3; ++b) {
                            zc rb = r[IXA(b, n, m, N) + 3 * NN * sc];
                            w->Omk[IXAB(i, b, n, m, N)] += phA * I * dRc[i] * rb;
                            w->Omk[IXAB(i, b, n, m, N)] -= phA * I * dRc[b] * ri;
                        }
                    }
                }
            }
    }
}

static void ft_R_to_k(const oracle_model *md, const double kpt[3], ws_t *w) {
    ft_zero(md->n_wf, w);
    ft_accum(md, kpt, w, 0, md->n_R);
}

/* ---------------- W -> H gauge (src/wann_interp.f90:465-658) ---------------- */
static int gauge_trafo(const oracle_model *md, ws_t *w, zc *Abar_out) {
    const int N = w->N;
    const size_t NN = (size_t)N * N;
    const int use_pos = (md->r != 0);
    zc *U = w->U;
    for (int a = 0; a < 3; ++a) {
        /* velocities: tmp = H_a U ; M = U^dag tmp (:520-528) */
        get_comp(N, w->Hka, 3, a, w->Min);
        zmm(N, w->Min, U, w->tmp);
        zmm_dagA(N, U, w->tmp, w->Min);
        put_comp(N, w->Hka, 3, a, w->Min);
        if (use_pos) {
            /* connection, D1 fixed: A_bar = U^dag A U */
            get_comp(N, w->Aka, 3, a, w->Min);
            zmm(N, w->Min, U, w->tmp);
            zmm_dagA(N, U, w->tmp, w->Min);
            put_comp(N, w->Aka, 3, a, w->Min);
            for (int b = 0; b < 3; ++b) { /* curvature (:538-544) */
                get_comp(N, w->Omk, 9, a + 3 * b, w->Min);
                zmm_dagA(N, U, w->Min, w->tmp);
                zmm(N, w->tmp, U, w->Min);
                put_comp(N, w->Omk, 9, a + 3 * b, w->Min);
            }
        }
    }
    if (!use_pos) return 0;
    if (Abar_out) memcpy(Abar_out, w->Aka, 3 * NN * sizeof(zc));
    /* covariant derivative (:565-617) */
    memset(w->D, 0, 3 * NN * sizeof(zc));
    for (int m = 0; m < N; ++m)
        for (int n = 0; n < N; ++n)
            if (n > m) {
                double ed = w->E[m] - w->E[n];
                if (fabs(ed) > md->kubo_tol)
                    for (int a = 0; a < 3; ++a) {
                        w->D[IXA(a, n, m, N)] = w->Hka[IXA(a, n, m, N)] / ed;
                        w->D[IXA(a, m, n, N)] = w->Hka[IXA(a, m, n, N)] / (-ed);
                    }
            }
    /* conn_gaugeTrafo (:620-633) */
    for (size_t i = 0; i < 3 * NN; ++i) w->Aka[i] += I * w->D[i];
    /* curv_gaugeTrafo (:636-658); semantics 0 uses A^H (D4), 1 uses A_bar */
    const zc *Ause = (md->semantics == 0 || !Abar_out) ? w->Aka : Abar_out;
    zc *Da = malloc(NN * sizeof(zc)), *Db = malloc(NN * sizeof(zc));
    zc *Xa = malloc(NN * sizeof(zc)), *Xb = malloc(NN * sizeof(zc));
    zc *Om = malloc(NN * sizeof(zc)), *P = malloc(NN * sizeof(zc)), *Q = malloc(NN * sizeof(zc));
    if (!Da || !Db || !Xa || !Xb || !Om || !P || !Q) return -1;
    for (int b = 0; b < 3; ++b)
        for (int a = 0; a < 3; ++a) {
            get_comp(N, w->Omk, 9, a + 3 * b, Om);
            get_comp(N, w->D, 3, a, Da);
            get_comp(N, w->D, 3, b, Db);
            get_comp(N, Ause, 3, a, Xa);
            get_comp(N, Ause, 3, b, Xb);
            /* Om -= [D_a, A_b] */
            zmm(N, Da, Xb, P); zmm(N, Xb, Da, Q);
            for (size_t i = 0; i < NN; ++i) Om[i] -= (P[i] - Q[i]);
            /* Om += [D_b, A_a] */
            zmm(N, Db, Xa, P); zmm(N, Xa, Db, Q);
            for (size_t i = 0; i < NN; ++i) Om[i] += (P[i] - Q[i]);
            /* Om -= i [D_a, D_b] */
            zmm(N, Da, Db, P); zmm(N, Db, Da, Q);
            for (size_t i = 0; i < NN; ++i) Om[i] -= I * (P[i] - Q[i]);
            put_comp(N, w->Omk, 9, a + 3 * b, Om);
        }
    free(Da); free(Db); free(Xa); free(Xb); free(Om); free(P); free(Q);
    return 0;
}

/* get_velo (src/wann_interp.f90:406-444) with D2 position V_nn = H_nn */
static void get_velo(const oracle_model *md, ws_t *w, const zc *Abar) {
    const int N = w->N;
    const size_t NN = (size_t)N * N;
    if (md->r) {
        const zc *Av = (md->semantics == 0 || !md->do_gauge_trafo || !Abar) ? w->Aka : Abar;
        for (int m = 0; m < N; ++m)
            for (int n = 0; n < N; ++n) {
                if (n > m) {
                    zc ced = I * (w->E[m] - w->E[n]);
                    for (int a = 0; a < 3; ++a) {
                        w->V[IXA(a, n, m, N)] = w->Hka[IXA(a, n, m, N)] - ced * Av[IXA(a, n, m, N)];
                        w->V[IXA(a, m, n, N)] = w->Hka[IXA(a, m, n, N)] + ced * Av[IXA(a, m, n, N)];
                    }
                }
            }
        for (int n = 0; n < N; ++n)
            for (int a = 0; a < 3; ++a) w->V[IXA(a, n, n, N)] = w->Hka[IXA(a, n, n, N)];
    } else {
        memcpy(w->V, w->Hka, 3 * NN * sizeof(zc));
    }
}

static double fd_stat(double e_band, double e_fermi, double T_kelvin) { /* src/statistics.f90:41-62 */
    if (T_kelvin > MIN_TEMP) return 1.0 / (1.0 + exp((e_band - e_fermi) / (KB_EH_K * T_kelvin)));
    return (e_band < e_fermi) ? 1.0 : 0.0;
}

/* full per-k interpolation (src/wann_interp.f90:56-108) */
/* get_wann_interp after FT_R_to_k: eigensolve, gauge transformation, velocity */
static int interp_after_ft(const oracle_model *md, ws_t *w, zc *Abar) {
    const int N = w->N;
    memcpy(w->U, w->Hk, (size_t)N * N * sizeof(zc));
    if (!g_zheevd) return -2;
    int n = N, lwork = N * N + 2 * N, lrwork = 2 * N * N + 5 * N + 1, liwork = 5 * N + 3, info = 0;
    g_zheevd("V", "U", &n, w->U, &n, w->E, w->work, &lwork, w->rwork, &lrwork, w->iwork, &liwork, &info, 1, 1);
    if (info != 0) return -3;
    if (md->do_gauge_trafo) {
        if (gauge_trafo(md, w, Abar) != 0) return -1;
    }
    get_velo(md, w, (md->do_gauge_trafo && md->r) ? Abar : 0);
    return 0;
}

static int interp_k(const oracle_model *md, const double kpt[3], ws_t *w, zc *Abar) {
    ft_R_to_k(md, kpt, w);
    return interp_after_ft(md, w, Abar);
}

/* band sums for one k, added into the given accumulators */
static void band_sums(const oracle_model *md, const oracle_job *jb, ws_t *w, double *Ne, double *ahc,
                      double *mic, double *mlc, double *mcs, double *kic, double *klc, double *kcs, zc *vah, zc *koh) {
    const int N = w->N, nE = jb->n_eF, nv = jb->valence_bands;
    const double tol = md->kubo_tol;
    const zc *V = w->V;
    const double *E = w->E;
    for (int n = 0; n < N; ++n)
        for (int e = 0; e < nE; ++e) {
            double f = fd_stat(E[n], jb->ef_lst[e], jb->T_kelvin);
            w->fd[e + nE * n] = f;
            Ne[e] += f;
        }
    if (jb->do_mep) {
        /* mep_niu_IC (src/mep_niu.f90:102-159) */
        for (int n0 = 0; n0 < nv; ++n0)
            for (int m = 0; m < N; ++m)
                for (int n = 0; n < N; ++n) {
                    if (n == n0 || m == n0) continue;
                    double den = (E[n0] - E[n]) * (E[n0] - E[n]) * (E[n0] - E[m]);
                    if (!(fabs(den) > tol)) continue;
                    for (int j = 0; j < 3; ++j)
                        for (int k = 0; k < 3; ++k)
                            for (int l = 0; l < 3; ++l) {
                                double pf = -(double)levi(j, k, l);
                                if (fabs(pf) > 1e-1)
                                    for (int i = 0; i < 3; ++i) {
                                        double vn = creal(V[IXA(i, n0, n, N)] * V[IXA(k, n, m, N)] * V[IXA(l, m, n0, N)]);
                                        mic[i + 3 * j + 9 * n0] += pf * vn / den;
                                    }
                            }
                }
        /* mep_niu_LC (src/mep_niu.f90:47-99) */
        for (int n0 = 0; n0 < nv; ++n0)
            for (int n = 0; n < N; ++n) {
                if (n == n0) continue;
                double d = E[n0] - E[n];
                double den = d * d * d;
                if (!(fabs(den) > tol)) continue;
                for (int j = 0; j < 3; ++j)
                    for (int k = 0; k < 3; ++k)
                        for (int l = 0; l < 3; ++l) {
                            double pf = (double)levi(j, k, l);
                            if (fabs(pf) > 1e-1)
                                for (int i = 0; i < 3; ++i) {
                                    double vn = creal(V[IXA(i, n0, n, N)] * V[IXA(k, n, n0, N)] * V[IXA(l, n0, n0, N)]);
                                    mlc[i + 3 * j + 9 * n0] += pf * vn / den;
                                }
                        }
            }
        /* mep_niu_CS (src/mep_niu.f90:20-44) */
        if (md->r)
            for (int n0 = 0; n0 < nv; ++n0) {
                zc om[3] = {0, 0, 0};
                for (int c = 0; c < 3; ++c)
                    for (int b = 0; b < 3; ++b)
                        for (int a = 0; a < 3; ++a) om[c] += (double)levi(a, b, c) * w->Omk[IXAB(a, b, n0, n0, N)];
                zc dp = 0;
                for (int c = 0; c < 3; ++c) dp += conj(w->Aka[IXA(c, n0, n0, N)]) * om[c];
                for (int i = 0; i < 3; ++i) mcs[i + 3 * i + 9 * n0] += 0.5 * creal(dp);
            }
    }
    if (jb->do_kubo) {
        /* kubo_mep_CS (src/kubo_mep.f90:16-47) */
        if (md->r)
            for (int n0 = 0; n0 < N; ++n0) {
                zc om[3] = {0, 0, 0};
                for (int c = 0; c < 3; ++c)
                    for (int b = 0; b < 3; ++b)
                        for (int a = 0; a < 3; ++a) om[c] += (double)levi(a, b, c) * w->Omk[IXAB(a, b, n0, n0, N)];
                zc dp = 0;
                for (int c = 0; c < 3; ++c) dp += conj(w->Aka[IXA(c, n0, n0, N)]) * om[c];
                for (int e = 0; e < nE; ++e) {
                    double v = 0.5 * w->fd[e + nE * n0] * creal(dp);
                    for (int i = 0; i < 3; ++i) kcs[i + 3 * i + 9 * e] += v;
                }
            }
        /* kubo_mep_LC (src/kubo_mep.f90:51-97) */
        for (int n0 = 0; n0 < N; ++n0)
            for (int n = 0; n < N; ++n) {
                if (n == n0) continue;
                double d = E[n0] - E[n];
                double den = d * d * d;
                double v[9] = {0};
                for (int j = 0; j < 3; ++j)
                    for (int k = 0; k < 3; ++k)
                        for (int l = 0; l < 3; ++l)
                            for (int i = 0; i < 3; ++i)
                                v[i + 3 * j] += (double)levi(j, k, l) *
                                                creal(V[IXA(i, n0, n, N)] * V[IXA(k, n, n0, N)] * V[IXA(l, n0, n0, N)]);
                for (int e = 0; e < nE; ++e)
                    for (int q = 0; q < 9; ++q) klc[q + 9 * e] += v[q] * w->fd[e + nE * n0] / den;
            }
        /* kubo_mep_IC (src/kubo_mep.f90:100-149) */
        for (int n0 = 0; n0 < N; ++n0)
            for (int m = 0; m < N; ++m)
                for (int n = 0; n < N; ++n) {
                    if (n == n0 || m == n0) continue;
                    double den = (E[n0] - E[m]) * (E[n0] - E[n]) * (E[n0] - E[n]);
                    double v[9] = {0};
                    for (int j = 0; j < 3; ++j)
                        for (int l = 0; l < 3; ++l)
                            for (int k = 0; k < 3; ++k)
                                for (int i = 0; i < 3; ++i)
                                    v[i + 3 * j] -= (double)levi(j, k, l) *
                                                    creal(V[IXA(i, n0, n, N)] * V[IXA(k, n, m, N)] * V[IXA(l, m, n0, N)]);
                    for (int e = 0; e < nE; ++e)
                        for (int q = 0; q < 9; ++q) kic[q + 9 * e] += v[q] * w->fd[e + nE * n0] / den;
                }
    }
    if (jb->do_ahc) {
        /* kubo_ahc_tens (src/kubo.f90:37-78) */
        for (int n = 0; n < N; ++n) {
            double curv[9] = {0};
            for (int np = 0; np < N; ++np) {
                if (np == n) continue;
                double d = E[np] - E[n];
                for (int j = 0; j < 3; ++j)
                    for (int i = 0; i < 3; ++i)
                        curv[i + 3 * j] -= 2.0 * cimag(V[IXA(i, n, np, N)] * V[IXA(j, np, n, N)]) / (d * d);
            }
            for (int e = 0; e < nE; ++e)
                for (int q = 0; q < 9; ++q) ahc[q + 9 * e] -= curv[q] * w->fd[e + nE * n];
        }
        if (jb->n_hw > 0 && jb->hw_lst) {
            const int nW = jb->n_hw;
            const zc ieta = I * jb->eta_smr;
            /* velo_ahc_tens (src/kubo.f90:86-140) */
            for (int n = 0; n < N; ++n)
                for (int np = 0; np < N; ++np) {
                    if (np == n) continue;
                    const double dE2 = (E[n] - E[np]) * (E[n] - E[np]);
                    double v[9];
                    for (int j = 0; j < 3; ++j)
                        for (int i = 0; i < 3; ++i) v[i + 3 * j] = cimag(V[IXA(i, n, np, N)] * V[IXA(j, np, n, N)]);
                    for (int h = 0; h < nW; ++h) {
                        const zc z = jb->hw_lst[h] + ieta;
                        const zc den = dE2 - z * z;
                        for (int e = 0; e < nE; ++e) {
                            const double df = w->fd[e + nE * n] - w->fd[e + nE * np];
                            for (int q = 0; q < 9; ++q) vah[q + 9 * (h + (size_t)nW * e)] += df * v[q] / den;
                        }
                    }
                }
            /* kubo_ohc_tens (src/kubo.f90:146-198), no degeneracy guard (D9) */
            for (int m = 0; m < N; ++m)
                for (int n = 0; n < N; ++n) {
                    if (m == n) continue;
                    const double dE = E[m] - E[n];
                    zc v[9];
                    for (int j = 0; j < 3; ++j)
                        for (int i = 0; i < 3; ++i) v[i + 3 * j] = V[IXA(i, n, m, N)] * V[IXA(j, m, n, N)];
                    for (int h = 0; h < nW; ++h) {
                        const zc den = dE * (dE - jb->hw_lst[h] - ieta);
                        for (int e = 0; e < nE; ++e) {
                            const double df = w->fd[e + nE * m] - w->fd[e + nE * n];
                            for (int q = 0; q < 9; ++q) koh[q + 9 * (h + (size_t)nW * e)] += I * v[q] / den * df;
                        }
                    }
                }
        }
    }
}

/* MP k-point of a 0-based linear index (src/k_space.f90:341-375) */
static void rel_kpt(const int32_t mp[3], int64_t ki, double k[3]) {
    int64_t q[3];
    q[0] = ki % mp[0] + 1;
    q[1] = (ki / mp[0]) % mp[1] + 1;
    q[2] = ki / ((int64_t)mp[0] * mp[1]) + 1;
    for (int i = 0; i < 3; ++i) k[i] = (2.0 * (double)q[i] - (double)mp[i] - 1.0) / (2.0 * (double)mp[i]);
}

/* Sum the k-loop body over k = k_begin + s*k_stride, s = 0..k_count-1 */
int oracle_run(const oracle_model *md, const oracle_job *jb, int64_t k_begin, int64_t k_count, int64_t k_stride,
               oracle_out *out, int nthreads) {
    const int N = md->n_wf, nE = jb->n_eF, nv = jb->valence_bands;
    if (N <= 0 || md->n_R <= 0 || nE <= 0 || nv < 0 || nv > N) return -1;
    if (!g_zheevd) return -2;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    const size_t sz_e = (size_t)nE, sz_9e = 9 * (size_t)nE, sz_9v = 9 * (size_t)(nv > 0 ? nv : 1);
    const int omega = jb->do_ahc && jb->n_hw > 0 && jb->hw_lst && out->velo_ahc && out->kubo_ohc;
    const size_t sz_w = omega ? 9 * (size_t)jb->n_hw * nE : 0;   /* complex elements per tensor */
    const size_t per = sz_e + 4 * sz_9e + 3 * sz_9v + 4 * sz_w;
    double *part = calloc((size_t)nthreads * per, sizeof(double));
    int64_t *cnt = calloc(nthreads, sizeof(int64_t));
    int err = 0;
    if (!part || !cnt) return -1;
#pragma omp parallel num_threads(nthreads)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        double *p = part + (size_t)t * per;
        double *Ne = p, *ahc = Ne + sz_e, *kic = ahc + sz_9e, *klc = kic + sz_9e, *kcs = klc + sz_9e;
        double *mic = kcs + sz_9e, *mlc = mic + sz_9v, *mcs = mlc + sz_9v;
        zc *vah = (zc *)(mcs + sz_9v), *koh = vah + sz_w;
        ws_t w = ws_alloc(N, nE);
        oracle_job jl = *jb;
        if (!omega) jl.n_hw = 0;
        zc *Abar = md->r ? calloc(3 * (size_t)N * N, sizeof(zc)) : 0;
#pragma omp for schedule(static)
        for (int64_t s = 0; s < k_count; ++s) {
            double k[3];
            rel_kpt(jb->mp_grid, k_begin + s * k_stride, k);
            int rc = interp_k(md, k, &w, Abar);
            if (rc != 0) {
#pragma omp atomic write
                err = rc;
                continue;
            }
            band_sums(md, &jl, &w, Ne, ahc, mic, mlc, mcs, kic, klc, kcs, vah, koh);
            cnt[t] += 1;
        }
        free(Abar);
        ws_free(&w);
    }
    /* deterministic merge in thread order */
    for (int t = 0; t < nthreads; ++t) {
        double *p = part + (size_t)t * per;
        double *Ne = p, *ahc = Ne + sz_e, *kic = ahc + sz_9e, *klc = kic + sz_9e, *kcs = klc + sz_9e;
        double *mic = kcs + sz_9e, *mlc = mic + sz_9v, *mcs = mlc + sz_9v;
        for (size_t i = 0; i < sz_e; ++i) out->Ne_sum[i] += Ne[i];
        for (size_t i = 0; i < sz_9e; ++i) {
            out->ahc[i] += ahc[i];
            out->kubo_mep_ic[i] += kic[i];
            out->kubo_mep_lc[i] += klc[i];
            out->kubo_mep_cs[i] += kcs[i];
        }
        for (size_t i = 0; i < 9 * (size_t)nv; ++i) {
            out->mep_ic[i] += mic[i];
            out->mep_lc[i] += mlc[i];
            out->mep_cs[i] += mcs[i];
        }
        const zc *vah = (const zc *)(mcs + sz_9v), *koh = vah + sz_w;
        for (size_t i = 0; i < sz_w; ++i) {
            out->velo_ahc[2 * i] += creal(vah[i]);
            out->velo_ahc[2 * i + 1] += cimag(vah[i]);
            out->kubo_ohc[2 * i] += creal(koh[i]);
            out->kubo_ohc[2 * i + 1] += cimag(koh[i]);
        }
        out->n_k += cnt[t];
    }
    free(part);
    free(cnt);
    return err;
}

/* The same sums with the reference's parallel structure (src/core.f90:165-270
 * around src/wann_interp.f90:206-241): a serial loop over k; inside each k the
 * Fourier sum runs over R on all threads, each thread summing a contiguous R
 * range into private matrices that are then added in thread order (the
 * reference's OpenMP array reduction); the eigensolve, gauge transformation
 * and band sums of that k run on one thread. */
int oracle_run_kserial(const oracle_model *md, const oracle_job *jb, int64_t k_begin, int64_t k_count,
                       int64_t k_stride, oracle_out *out, int nthreads) {
    const int N = md->n_wf, nE = jb->n_eF, nv = jb->valence_bands, nR = md->n_R;
    if (N <= 0 || nR <= 0 || nE <= 0 || nv < 0 || nv > N) return -1;
    if (!g_zheevd) return -2;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    const size_t NN = (size_t)N * N;
    const int omega = jb->do_ahc && jb->n_hw > 0 && jb->hw_lst && out->velo_ahc && out->kubo_ohc;
    oracle_job jl = *jb;
    if (!omega) jl.n_hw = 0;
    ws_t w = ws_alloc(N, nE);
    ws_t *tw = calloc(nthreads, sizeof(ws_t));
    zc *Abar = md->r ? calloc(3 * NN, sizeof(zc)) : 0;
    if (!tw) return -1;
    for (int t = 0; t < nthreads; ++t) tw[t] = ws_alloc(N, 1);
    int err = 0;
    for (int64_t s = 0; s < k_count && !err; ++s) {
        double k[3];
        rel_kpt(jb->mp_grid, k_begin + s * k_stride, k);
#pragma omp parallel num_threads(nthreads)
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            ft_zero(N, &tw[t]);
            ft_accum(md, k, &tw[t], (int)((int64_t)nR * t / nthreads), (int)((int64_t)nR * (t + 1) / nthreads));
        }
        ft_zero(N, &w);
        for (int t = 0; t < nthreads; ++t) {
            for (size_t i = 0; i < NN; ++i) w.Hk[i] += tw[t].Hk[i];
            for (size_t i = 0; i < 3 * NN; ++i) {
                w.Hka[i] += tw[t].Hka[i];
                w.Aka[i] += tw[t].Aka[i];
            }
            for (size_t i = 0; i < 9 * NN; ++i) w.Omk[i] += tw[t].Omk[i];
        }
        int rc = interp_after_ft(md, &w, Abar);
        if (rc != 0) {
            err = rc;
            break;
        }
        band_sums(md, &jl, &w, out->Ne_sum, out->ahc, out->mep_ic, out->mep_lc, out->mep_cs, out->kubo_mep_ic,
                  out->kubo_mep_lc, out->kubo_mep_cs, omega ? (zc *)out->velo_ahc : 0,
                  omega ? (zc *)out->kubo_ohc : 0);
        out->n_k += 1;
    }
    for (int t = 0; t < nthreads; ++t) ws_free(&tw[t]);
    free(tw);
    free(Abar);
    ws_free(&w);
    return err;
}

/* One k: E(N), V(3,N,N), A(3,N,N), Om(3,3,N,N) (complex, Fortran layout). */
int oracle_interp_k(const oracle_model *md, const double kpt[3], double *E, double *V, double *A, double *Om) {
    const int N = md->n_wf;
    const size_t NN = (size_t)N * N;
    ws_t w = ws_alloc(N, 1);
    zc *Abar = md->r ? calloc(3 * NN, sizeof(zc)) : 0;
    int rc = interp_k(md, kpt, &w, Abar);
    if (rc == 0) {
        memcpy(E, w.E, N * sizeof(double));
        memcpy(V, w.V, 3 * NN * sizeof(zc));
        if (A && md->r) memcpy(A, w.Aka, 3 * NN * sizeof(zc));
        if (Om && md->r) memcpy(Om, w.Omk, 9 * NN * sizeof(zc));
    }
    free(Abar);
    ws_free(&w);
    return rc;
}
