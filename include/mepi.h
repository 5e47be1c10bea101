/*
 * mepi.h -- C ABI of the GB300 (sm_103a) implementation of MEPinterp's
 * per-k-point Wannier-interpolation path (AHC + Niu MEP + Kubo MEP).
 *
 * The reference has no plugin or FFI layer: its boundary is the body of the
 * k-loop in src/core.f90:165-270, which calls get_wann_interp
 * (src/wann_interp.f90:56-108) and the band sums kubo_ahc_tens
 * (src/kubo.f90:37-78), mep_niu_IC/LC/CS (src/mep_niu.f90:20-159) and
 * kubo_mep_IC/LC/CS (src/kubo_mep.f90:16-149) once per k-point, adding into
 * the *_loc accumulators allocated in src/core.f90:610-691.  One mepi_run call
 * replaces that whole loop for one MPI rank: it returns the same unnormalised
 * local sums, so fermi_selector and integrate_over_k_space
 * (src/core.f90:276-292) run unchanged on top of it.
 *
 * Conventions
 *  - All arrays use the reference's Fortran (column-major, 1-based in Fortran)
 *    layout; complex numbers are interleaved (re, im) doubles.
 *  - Units are the reference's internal atomic units (Hartree, bohr), i.e.
 *    what read_tb_basis leaves in memory (src/file_io.f90:741, :790).
 *  - The caller owns every host buffer; the library owns its device state and
 *    copies the model to the GPU in mepi_create.
 *  - Every function returns 0 on success or a MEPI_ERR_* code; nothing exits
 *    the process (the reference calls `stop`; a Fortran shim maps a nonzero
 *    status to `stop`).
 *  - Threading: one context per host thread; calls are synchronous.
 */
#ifndef MEPI_H
#define MEPI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MEPI_OK 0
#define MEPI_ERR_ARG 1          /* bad shape, NULL pointer, bad option */
#define MEPI_ERR_CUDA 2         /* CUDA runtime error or no usable device */
#define MEPI_ERR_NOMEM 3        /* device allocation failed */
#define MEPI_ERR_EIG 4          /* Jacobi eigensolver hit its sweep cap */
#define MEPI_ERR_NONHERM 5      /* H(R) is not Hermitian: H(-R) != H(R)^dag */
#define MEPI_ERR_NONFINITE 6    /* NaN/Inf in the input model */
#define MEPI_ERR_SCRATCH 7      /* mepi_bandsum_noalloc: problem larger than its
                                   fixed scratch array */

/* semantics where the reference is not reproducible (see mepi_model) */
#define MEPI_SEM_REF 0
#define MEPI_SEM_PAPER 1

/* output mask (src/core.f90:198-230: do_mep, do_kubo, do_ahc) */
#define MEPI_OUT_AHC 1u
#define MEPI_OUT_MEP_NIU 2u
#define MEPI_OUT_KUBO_MEP 4u
#define MEPI_OUT_OPT_HALL 8u    /* velo_ahc_tens + kubo_ohc_tens (src/kubo.f90:86-198),
                                   which the reference computes with do_ahc
                                   (src/core.f90:221-230); needs n_hw >= 1 */

/* arithmetic form of the run */
#define MEPI_PREC_FP64 0   /* all-FP64 plain form */
#define MEPI_PREC_MIXED 1  /* FP32 per-k work with FP64 H(k), compensated
                              eigenpair refinement and velocity rotation, FP64
                              energies for every decision and FP64 k-sums;
                              k-points whose band gap falls below degen_gap
                              are rerun in FP64 */

typedef struct mepi_ctx mepi_ctx;

/* The tight-binding basis: what read_tb_basis (src/file_io.f90:800-860) and
 * init_parameters (src/input_paras.f90:79-293) leave in memory. */
typedef struct {
    int32_t n_wf;              /* number of Wannier functions N */
    int32_t n_R;               /* number of lattice vectors nR */
    const double *R_frac;      /* R_frac(3, n_R), lattice units */
    const double *H;           /* complex H_real(N, N, n_R), Hartree */
    const double *r;           /* complex r_real(3, N, N, n_R), bohr; NULL = no
                                  position operator (no A, Omega, CS terms) */
    const double *wf_centers;  /* wf_centers(3, N), lattice units; NULL selects
                                  the Wannier phase convention */
    double a_latt[9];          /* a_latt(3,3) column-major (row i = a_i) */
    int32_t do_gauge_trafo;    /* [wannInterp] doGaugeTrafo */
    int32_t use_cart_velo;     /* [wannInterp] use_cart_velo */
    int32_t semantics;         /* MEPI_SEM_REF: curvature and velocity from
                                  A^H = A_bar + iD as the reference computes
                                  them; MEPI_SEM_PAPER: from A_bar */
    double kubo_tol;           /* [Fermi] kuboTol */
} mepi_model;

/* One rank's share of the k-loop (src/core.f90:165-270). */
typedef struct {
    int32_t mp_grid[3];        /* Monkhorst-Pack mesh */
    int64_t k_begin;           /* first 0-based linear k index (kx fastest) */
    int64_t k_stride;          /* stride between owned k; mpi_ki_selector
                                  (src/mpi_comm.f90:80-99) = rank, nProcs */
    int64_t k_count;           /* number of k to process; < 0 = all owned */
    int32_t n_eF;              /* number of Fermi energies */
    const double *ef_lst;      /* ef_lst(n_eF), Hartree */
    double T_kelvin;           /* temperature; <= 1e-2 K means a step function */
    int32_t valence_bands;     /* [MEP] valence_bands (0..N) */
    uint32_t outputs;          /* MEPI_OUT_* mask */
    int32_t precision;         /* MEPI_PREC_* */
    int64_t chunk_k;           /* k-points per device chunk; 0 = automatic */
    double degen_gap;          /* MEPI_PREC_MIXED only: minimum band gap (Ha)
                                  for the FP32 per-k path; < 0 = default
                                  (3e-3 Ha) */
    int32_t n_hw;              /* MEPI_OUT_OPT_HALL: number of photon energies */
    const double *hw_lst;      /* hw_lst(n_hw), Hartree ([Laser] get_linspace) */
    double eta_smr;            /* [Fermi] eta_smearing, Hartree: the reference's
                                  i_eta_smr = i * eta_smr */
    const int64_t *k_list;     /* optional: k_count 0-based linear mesh indices
                                  (kx fastest) to run instead of k_begin,
                                  k_stride -- e.g. the cells an adaptive
                                  refinement picked; NULL = the stride rule */
} mepi_job;

/* Unnormalised local sums, like the reference's *_loc arrays
 * (src/core.f90:610-691).  Each pointer may be NULL when its output is not
 * requested; buffers are overwritten (not accumulated into). */
typedef struct {
    double *Ne_sum;            /* Ne_loc_sum(n_eF) */
    double *ahc;               /* kubo_ahc_loc(3,3,n_eF) */
    double *mep_ic;            /* mep_bands_ic_loc(3,3,valence_bands) */
    double *mep_lc;            /* mep_bands_lc_loc(3,3,valence_bands) */
    double *mep_cs;            /* mep_bands_cs_loc(3,3,valence_bands) */
    double *kubo_mep_ic;       /* kubo_mep_ic_loc(3,3,n_eF) */
    double *kubo_mep_lc;       /* kubo_mep_lc_loc(3,3,n_eF) */
    double *kubo_mep_cs;       /* kubo_mep_cs_loc(3,3,n_eF) */
    int64_t n_k_done;          /* n_ki_loc */
    int64_t n_k_fp64;          /* MEPI_PREC_MIXED: k-points rerun in FP64 */
    int32_t eig_max_sweeps;    /* largest Jacobi sweep count seen */
    double *velo_ahc;          /* MEPI_OUT_OPT_HALL: velo_ahc_loc(3,3,n_hw,n_eF)
                                  complex, as (re, im) pairs */
    double *kubo_ohc;          /* MEPI_OUT_OPT_HALL: kubo_ohc_loc(3,3,n_hw,n_eF)
                                  complex, as (re, im) pairs */
    double *perk;              /* optional per-k output, perk(4, n_k) in the
                                  job's k order: the (y,z), (z,x), (x,y)
                                  entries of the k-point's kubo_ahc_tens term
                                  at ef_lst(1), and the band gap across
                                  ef_lst(1) (Hartree) */
} mepi_acc;

/* Device time of each stage of the last mepi_run (CUDA events on the
 * library's stream), milliseconds, with launch counts. */
typedef struct {
    double ft_ms;              /* Fourier sums (separable, SIMT FP64 or tensor-core GEMM) */
    double phase_ms;           /* mixed form: phase-operand generation */
    double fth_ms;             /* mixed form: FP64 Fourier sum of H(k) alone */
    double eig_ms;             /* Jacobi eigensolver */
    double refine_ms;          /* mixed form: FP64 eigenpair refinement */
    double rot_ms, gauge_ms, bandsum_ms, reduce_ms;
    double total_ms;           /* sum of the stage times */
    double run_ms;             /* whole call, first launch to last copy back */
    int32_t ft_launches, phase_launches, fth_launches, eig_launches, refine_launches, rot_launches,
        gauge_launches, bandsum_launches, reduce_launches;
    int64_t n_k;               /* k-points of the run */
    int64_t h2d_bytes;         /* host->device bytes since mepi_create */
    int64_t d2h_bytes;         /* device->host bytes since mepi_create */
    double plan_ms;            /* host wall time building the separable-sum slabs
                                  (0 when a run reuses the slabs of its mesh) */
} mepi_timing;

/* Launch shapes of the per-k kernels of one context.  No counterpart in the
 * reference.  0 selects the built-in choice. */
typedef struct {
    int32_t jacobi_threads;    /* threads per eigensolver CTA: 64, 128 or 256 */
    int32_t jacobi_kblock;     /* k-points per eigensolver CTA, warm-started in turn */
    int64_t chunk_k;           /* k-points per device chunk (a job's chunk_k > 0 wins) */
    double k_per_s;            /* mepi_autotune: the measured rate of this choice */
} mepi_tuning;

/* Replaces read_tb_basis's arrays being handed to get_wann_interp
 * (src/core.f90:144, :179-182): validates and uploads the model. */
int mepi_create(mepi_ctx **out, const mepi_model *m);

/* Replaces the k-loop body src/core.f90:165-270 for one rank. */
int mepi_run(mepi_ctx *ctx, const mepi_job *job, mepi_acc *out);

/* Per-k results of get_wann_interp (src/wann_interp.f90:56-108) for a list of
 * k-points given in lattice units (kpts(3, n_k)): eigenvalues en_k(N, n_k),
 * velocities V_ka(3, N, N, n_k) complex; A_diag(3, N, n_k) and
 * Om_diag(3, 3, N, n_k) complex hold the band-diagonal connection and
 * curvature (the parts the band sums consume); either may be NULL. */
int mepi_interp_k(mepi_ctx *ctx, int32_t precision, int64_t n_k, const double *kpts,
                  double *en_k, double *V_ka, double *A_diag, double *Om_diag);

/* Device time per stage of the last mepi_run. */
int mepi_get_timing(const mepi_ctx *ctx, mepi_timing *t);

/* Autotuner.  No counterpart in the reference.  Times the candidate launch
 * shapes (eigensolver threads 64/128/256, warm-start run 4/8/16, chunk 16K/64K
 * k-points) on the first sample_k k-points of the job (<= 0: 32768), keeps the
 * fastest in the context and records it for the contexts created later in
 * this process with the same device, band count, R count and stack blocks. */
int mepi_autotune(mepi_ctx *ctx, const mepi_job *job, int64_t sample_k, mepi_tuning *best);
int mepi_set_tuning(mepi_ctx *ctx, const mepi_tuning *t);
int mepi_get_tuning(const mepi_ctx *ctx, mepi_tuning *t);

/* Device-memory limit of a context (no counterpart in the reference; 0, the
 * default, = half the free memory for the separable Fourier slabs and 8 GB --
 * 3 GB in the FP64 form -- for the per-chunk buffers).  With a limit, both
 * take at most half of it each: the chunk shrinks, and the slabs of a large
 * mesh are built for one range of qx after the other during the run.
 * Results do not depend on the limit. */
int mepi_set_mem_limit(mepi_ctx *ctx, uint64_t bytes);
/* Free the context's cached run buffers (separable slabs, chunk buffers);
 * the next run rebuilds them.  For callers that keep many contexts and run
 * them in turn.  No counterpart in the reference. */
int mepi_trim(mepi_ctx *ctx);

/* Batched form.  No counterpart in the reference, where each model is a
 * separate run.  n (context, job) pairs -- models of different band and R
 * counts, each with its own mesh, Fermi sweep and precision -- run as ONE
 * CUDA graph: every context's chunk pipeline is captured on its own stream
 * (independent models overlap on the GPU) and the graph is launched once.
 * The FP64 reruns of the mixed form, the reductions and the copies back
 * follow per context.  The contexts share 80% of the free device memory
 * (each within its own mepi_set_mem_limit as well).  All contexts must be on the same device.  graph_ms
 * (optional) receives the device time of the graph launch.  Results equal
 * those of n separate mepi_run calls. */
int mepi_run_batch(int32_t n, mepi_ctx *const *ctxs, const mepi_job *jobs, mepi_acc *accs, double *graph_ms);

/* Band sums without any device allocation.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory when they need the sums: a
 * host code that gives all device memory to its own pool at start-up, a job
 * held to a fixed device-memory budget, or a loop that cannot take the
 * latency and implicit synchronisation of cudaMalloc.  The caller already
 * holds, in device memory, the energies and velocity matrices of n_k
 * k-points (for instance from its own interpolation) and gets back the same
 * unnormalised sums mepi_run accumulates:
 *   en_k     device, n_k x n_wf FP64 eigenvalues (ascending per k-point)
 *   V        device, complex128 as (re, im) pairs, element (k, a, n, m) at
 *            ((k*3 + a)*n_wf + n)*n_wf + m: the velocity matrices V_ka
 *   csv      device, n_k x n_wf Chern-Simons per-band values
 *            0.5 Re(sum_c conj(A_c(n,n)) om_c(n)), or NULL for none
 *   ef_lst   device, n_eF Fermi energies (Hartree)
 *   sums     device, 37*n_eF + 27*valence_bands doubles, written (not added to)
 *            in the order Ne_sum(n_eF), ahc(3,3,n_eF), kubo_mep_ic(3,3,n_eF),
 *            kubo_mep_lc, kubo_mep_cs, mep_ic(3,3,valence_bands), mep_lc, mep_cs
 *   stream   a cudaStream_t, or NULL for the default stream; the work is
 *            enqueued there and the call returns without synchronising.
 * Its scratch is one fixed 4 MiB device array in the library (held by every
 * GPU that loads the library until the process exits), used as 152 slices of
 * 37*n_eF + 27*valence_bands doubles: problems with
 * 37*n_eF + 27*valence_bands > 3449 are rejected with MEPI_ERR_SCRATCH.  All
 * calls share that array, so calls whose work overlaps on the GPU (on
 * different streams, or from several host threads) race; serialise them.  The
 * first call on each device (and the first after that device's context is
 * replaced, e.g. by cudaDeviceReset) looks up the array's device address; make
 * that first call before capturing any stream.  Only the outputs bits
 * MEPI_OUT_AHC, MEPI_OUT_MEP_NIU and MEPI_OUT_KUBO_MEP are honoured; any other
 * bit is rejected with MEPI_ERR_ARG, as are a non-finite T_kelvin or kubo_tol.
 * ef_lst lives in device memory and is not validated. */
int mepi_bandsum_noalloc(int32_t n_wf, int64_t n_k, const double *en_k, const double *V, const double *csv,
                         int32_t n_eF, const double *ef_lst, double T_kelvin, int32_t valence_bands,
                         uint32_t outputs, double kubo_tol, double *sums, void *stream);

/* Frees the context and its device memory. */
int mepi_destroy(mepi_ctx *ctx);

/* Static message for a status code. */
const char *mepi_strerror(int status);

/* Library version string. */
const char *mepi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MEPI_H */
