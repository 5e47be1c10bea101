// C ABI of libmepi_gb300 (declared in include/mepi.h).
//
// mepi_create  validates the tight-binding basis (shapes, finiteness,
//              H(-R) = H(R)^dag) and uploads the Fourier stack S[R][pair][blk]
//              (see mepi_internal.cuh) built on the host in FP64.
// mepi_run     replaces the k-loop of src/core.f90:165-270 for one rank: the
//              owned k-points are streamed through the device in chunks
//              (FT -> eigensolve -> rotation -> gauge/velocity -> band sums),
//              the band sums accumulate into per-CTA FP64 slices that persist
//              across chunks, and one fixed-order reduction produces the
//              reference's *_loc sums.  In the mixed form the chunk runs in
//              FP32 and every k-point whose Jacobi did not converge or whose
//              smallest band gap is below degen_gap is skipped there and rerun
//              through the FP64 pipeline afterwards.
#include <algorithm>
#include <array>
#include <mutex>
#include <map>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/mepi.h"
#include "ft_tc.cuh"
#include "mepi_internal.cuh"

using namespace mepi;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b) {
        if (b <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename X> X* as() const { return reinterpret_cast<X*>(p); }
};

struct StageEv {
    cudaEvent_t a, b;
    int stage;
};

enum { ST_FT = 0, ST_PHASE, ST_FTH, ST_EIG, ST_REFINE, ST_ROT, ST_GAUGE, ST_BAND, ST_RED, ST_RUN, ST_N };

}  // namespace

struct mepi_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    DevModel dm{};
    int N = 0, nR = 0, nb = 0;
    double a_latt[9];
    DevBuf S, R, tau;
    // per-chunk work buffers
    DevBuf W, E, E64, H64, U, Ulo, HA, OD, V, CSV, ODH, flags, klist, kpts, partials, out, counters;
    // explicit k lists (mepi_job.k_list) and the per-k output (mepi_acc.perk)
    DevBuf jlist, kpos, rpos, perk;
    std::vector<int64_t> kpos_host;     // job position of each kcol_host entry
    int* h_flags = nullptr;  // pinned
    size_t h_flags_cap = 0;
    std::vector<StageEv> events;
    size_t ev_used = 0;
    mepi_timing timing{};
    int64_t h2d = 0, d2h = 0;           // host<->device byte counters
    std::vector<cplx<double>> S_host;  // FP64 stack, kept to build the tensor-core operands
    TcPlan tc;
    int ft_pref = 0;                    // MEPI_FT: 0 auto (separable when possible), 1 tensor core, 2 SIMT
    int rot_pref = 0;                   // MEPI_ROT: 0 auto (tensor cores in the mixed form), 2 SIMT
    int jacobi_warp = 1;                // FP32 Jacobi for N <= 32: register-resident warp form (MEPI_JACOBI=smem: CTA form)
    float jacobi_theta = 0.f;           // FP32 Jacobi: rotate a pair while |M_pq| > theta |M_pp - M_qq| (0: to the FP32 floor)
    std::vector<double> R_host;         // lattice vectors, kept for the separable plan
    SepPlan sep;                        // separable-sum slabs of the current mesh
    bool sep_active = false;            // this run's chunks take the separable sums
    double plan_ms = 0.0;
    // k-points of the run in (qx, qy)-column order, for slab reuse
    DevBuf kcol;
    std::vector<int64_t> kcol_host;
    std::vector<int64_t> kslab;         // kcol_host index where each qx slab starts (+ the end)
    int kslab_nqx = 0;                  // the slab width kslab was made for
    int64_t kcol_key[6] = {-1, -1, -1, -1, -1, -1};
    // launch shapes picked by mepi_autotune (0 = the built-in choice)
    mepi_tuning tune{};
    // state of the current run between its phases (prepare, enqueue, finish)
    struct Run {
        mepi_job job{};
        int64_t count = 0, chunk = 0;
        bool fp64 = true;
        double degen_gap = 3e-3;
        int n_hw = 0, n_cta = 0;
        AccLayout L{1, 0, 0};
        JobDev jb{};
        size_t run_ev = 0;
        bool perk = false;              // per-k output requested
        int64_t n_redo = 0;             // k-points rerun in FP64
        // the FP64 reruns between finish_prepare and finish_launch
        std::vector<int64_t> redo, redo_pos, rslab;
        int64_t rchunk = 0;
        bool sep_keep = false;
        bool in_reruns = false;         // the FP64 reruns are being enqueued (scattered k-points)
    } run;
    double* h_out = nullptr;            // pinned copy-back of the reduced sums and counters
    size_t h_out_cap = 0;
    bool timed = true;                  // per-stage CUDA events (off inside a graph capture)
    size_t mem_budget = 0;              // device bytes for slabs + chunk buffers (0: the defaults)
    size_t mem_limit = 0;               // the caller's limit (mepi_set_mem_limit)
};

namespace {

#define CK(x)                                         \
    do {                                              \
        cudaError_t _e = (x);                         \
        if (_e != cudaSuccess) return MEPI_ERR_CUDA;  \
    } while (0)

#define CKM(x)                                                                       \
    do {                                                                             \
        cudaError_t _e = (x);                                                        \
        if (_e == cudaErrorMemoryAllocation) { cudaGetLastError(); return MEPI_ERR_NOMEM; } \
        if (_e != cudaSuccess) return MEPI_ERR_CUDA;                                 \
    } while (0)

constexpr size_t kNoEvent = ~(size_t)0;
int stage_begin(mepi_ctx* c, int stage, size_t* idx) {
    if (!c->timed) {
        *idx = kNoEvent;
        return 0;
    }
    if (c->ev_used == c->events.size()) {
        StageEv ev{};
        CK(cudaEventCreate(&ev.a));
        CK(cudaEventCreate(&ev.b));
        c->events.push_back(ev);
    }
    *idx = c->ev_used++;
    c->events[*idx].stage = stage;
    CK(cudaEventRecord(c->events[*idx].a, c->stream));
    return 0;
}
int stage_end(mepi_ctx* c, size_t idx) {
    if (idx == kNoEvent) return 0;
    CK(cudaEventRecord(c->events[idx].b, c->stream));
    return 0;
}

#define STAGE(st, call)                                   \
    do {                                                  \
        size_t _i;                                        \
        int _r = stage_begin(ctx, st, &_i);               \
        if (_r) return _r;                                \
        CK(call);                                         \
        _r = stage_end(ctx, _i);                          \
        if (_r) return _r;                                \
    } while (0)

bool finite_all(const double* p, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(p[i])) return false;
    return true;
}

template <typename T>
size_t per_k_bytes(int N, int nb) {
    size_t NN = (size_t)N * N;
    return sizeof(cplx<T>) * (nb * NN + NN + 6 * NN + 3 * N + 3 * NN + 3 * N) + sizeof(T) * 2 * N + sizeof(int) +
           sizeof(int64_t) + sizeof(double) * N +
           (sizeof(T) == 4 ? (sizeof(cplx<double>) + sizeof(cplx<float>)) * NN : 0);
}

template <typename T>
int ensure_chunk(mepi_ctx* ctx, int64_t chunk) {
    const size_t NN = (size_t)ctx->N * ctx->N, N = ctx->N;
    CKM(ctx->W.ensure(chunk * ctx->nb * NN * sizeof(cplx<T>)));
    CKM(ctx->E.ensure(chunk * N * sizeof(T)));
    CKM(ctx->E64.ensure(chunk * N * sizeof(double)));
    if (sizeof(T) == 4) CKM(ctx->H64.ensure(chunk * NN * sizeof(float4)));
    CKM(ctx->U.ensure(chunk * NN * sizeof(cplx<T>)));
    if (sizeof(T) == 4) CKM(ctx->Ulo.ensure(chunk * NN * sizeof(cplx<float>)));   // refined vectors' low parts
    CKM(ctx->HA.ensure(chunk * 6 * NN * sizeof(cplx<T>)));
    CKM(ctx->OD.ensure(chunk * 3 * N * sizeof(cplx<T>)));
    CKM(ctx->V.ensure(chunk * 3 * NN * sizeof(cplx<T>)));
    CKM(ctx->CSV.ensure(chunk * N * sizeof(T)));
    CKM(ctx->flags.ensure(chunk * sizeof(int)));
    return 0;
}

// device bytes of a context's separable slabs and per-chunk buffers
size_t run_buffer_bytes(const mepi_ctx* ctx) {
    size_t b = ctx->sep.dev_bytes;
    for (const DevBuf* d : {&ctx->W, &ctx->E, &ctx->E64, &ctx->H64, &ctx->U, &ctx->Ulo, &ctx->HA, &ctx->OD, &ctx->V, &ctx->CSV,
                            &ctx->flags})
        b += d->bytes;
    return b;
}

void release_run_buffers(mepi_ctx* ctx) {
    cudaStreamSynchronize(ctx->stream);
    for (DevBuf* d : {&ctx->W, &ctx->E, &ctx->E64, &ctx->H64, &ctx->U, &ctx->Ulo, &ctx->HA, &ctx->OD, &ctx->V, &ctx->CSV,
                      &ctx->flags})
        d->release();
    sep_plan_free(ctx->sep);
}

// One chunk of k-points through FT -> eig (-> FP64 refinement) -> rot ->
// gauge (-> bandsum).  The band kernels always consume FP64 energies: the
// FP64 path's Jacobi writes them directly; the mixed path refines the FP32
// eigenpairs against an FP64 H(k) first.
template <typename T>
int run_chunk(mepi_ctx* ctx, const KRange& kr, const JobDev* jb, int n_cta, double degen_gap, bool want_flags,
              bool bandsum, cplx<T>* odh) {
    const int64_t nk = kr.count;
    int* counters = ctx->counters.as<int>();
    const bool mixed = sizeof(T) == 4;
    int* flags = want_flags ? ctx->flags.as<int>() : nullptr;
    const bool sep = ctx->sep_active && !kr.kpts && (mixed || ctx->sep.nbd == ctx->sep.nbk);
    if (sep) {
        STAGE(ST_FT, (launch_sep_w<T>(ctx->sep, ctx->dm, kr, ctx->W.as<cplx<T>>(), ctx->stream)));
    } else if (mixed && ctx->ft_pref != 2) {
        if (!ctx->tc.ready()) {
            int rc = tc_plan_init(ctx->tc, ctx->dm, ctx->S_host.data());
            if (rc) return rc;
            ctx->h2d += 2 * (int64_t)ctx->tc.ncolp * ctx->tc.Kp * sizeof(__half);
        }
        int rc = tc_plan_rows(ctx->tc, nk);
        if (rc) return rc;
        STAGE(ST_PHASE, launch_phase_split(ctx->tc, kr, ctx->stream));
        STAGE(ST_FT, launch_ft_tc(ctx->tc, kr, reinterpret_cast<cplx<float>*>(ctx->W.p), ctx->stream));
    } else {
        STAGE(ST_FT, (launch_ft_simt<T>(ctx->dm, kr, ctx->W.as<cplx<T>>(), ctx->stream)));
    }
    double* E64 = ctx->E64.as<double>();
    if (mixed) {
        // FP64 H(k), FP32 Jacobi on it, FP64 residual refinement of the eigenpairs
        float4* H64 = ctx->H64.as<float4>();
        if (sep)
            STAGE(ST_FTH, launch_sep_h64(ctx->sep, kr, H64, ctx->stream));
        else
            STAGE(ST_FTH, launch_ft_h64(ctx->dm, kr, H64, ctx->stream));
        STAGE(ST_EIG, (launch_eig<T>(ctx->N, nk, ctx->W.as<cplx<T>>(), ctx->nb, H64, ctx->E.as<T>(),
                                     ctx->U.as<cplx<T>>(), 40, counters, counters + 2, degen_gap, flags, ctx->stream,
                                     ctx->jacobi_warp == 2 ? 1 : ctx->tune.jacobi_threads, ctx->tune.jacobi_kblock,
                                     ctx->jacobi_theta, ctx->jacobi_warp != 0)));
        STAGE(ST_REFINE, launch_refine(ctx->N, nk, H64, reinterpret_cast<const float*>(ctx->E.p),
                                       reinterpret_cast<cplx<float>*>(ctx->U.p), ctx->Ulo.as<cplx<float>>(), E64,
                                       degen_gap, flags, ctx->stream));
    } else {
        // the reruns' k-points are scattered over the mesh: a warm start from the
        // previous one would not be a neighbour's, so one k-point per CTA (cold
        // starts, and every CTA of the few hundred to few thousand runs at once)
        STAGE(ST_EIG, (launch_eig<T>(ctx->N, nk, ctx->W.as<cplx<T>>(), ctx->nb, nullptr, reinterpret_cast<T*>(E64),
                                     ctx->U.as<cplx<T>>(), 40, counters, counters + 1, degen_gap, flags, ctx->stream,
                                     ctx->tune.jacobi_threads, ctx->run.in_reruns ? 1 : ctx->tune.jacobi_kblock)));
    }
    if (mixed && ctx->rot_pref == 0 && rot_tc_supported(ctx->dm)) {
        // tensor-core rotation; a timed-out wait raises counters[3]
        STAGE(ST_ROT, launch_rot_tc(ctx->dm, nk, reinterpret_cast<const cplx<float>*>(ctx->W.p),
                                    reinterpret_cast<const cplx<float>*>(ctx->U.p), ctx->Ulo.as<cplx<float>>(),
                                    reinterpret_cast<cplx<float>*>(ctx->HA.p), reinterpret_cast<cplx<float>*>(ctx->OD.p),
                                    counters + 3, ctx->stream));
    } else {
        STAGE(ST_ROT, (launch_rot<T>(ctx->dm, nk, ctx->W.as<cplx<T>>(), ctx->U.as<cplx<T>>(), ctx->HA.as<cplx<T>>(),
                                     ctx->OD.as<cplx<T>>(), ctx->stream)));
    }
    STAGE(ST_GAUGE, (launch_gauge<T>(ctx->dm, nk, E64, ctx->HA.as<cplx<T>>(), ctx->OD.as<cplx<T>>(),
                                     ctx->V.as<cplx<T>>(), ctx->CSV.as<T>(), odh, ctx->stream)));
    if (bandsum) {
        STAGE(ST_BAND, (launch_bandsum<T>(ctx->dm, *jb, nk, E64, ctx->V.as<cplx<T>>(), ctx->CSV.as<T>(), flags,
                                          ctx->partials.as<double>(), n_cta, ctx->stream)));
        if (jb->nW > 0)
            STAGE(ST_BAND, (launch_opt_hall<T>(ctx->dm, *jb, nk, E64, ctx->V.as<cplx<T>>(), flags,
                                               ctx->partials.as<double>(), n_cta, ctx->stream)));
    }
    return 0;
}

int collect_timing(mepi_ctx* ctx, int64_t nk) {
    mepi_timing t{};
    t.n_k = nk;
    for (size_t i = 0; i < ctx->ev_used; ++i) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->events[i].a, ctx->events[i].b));
        switch (ctx->events[i].stage) {
            case ST_FT: t.ft_ms += ms; t.ft_launches++; break;
            case ST_PHASE: t.phase_ms += ms; t.phase_launches++; break;
            case ST_FTH: t.fth_ms += ms; t.fth_launches++; break;
            case ST_EIG: t.eig_ms += ms; t.eig_launches++; break;
            case ST_REFINE: t.refine_ms += ms; t.refine_launches++; break;
            case ST_ROT: t.rot_ms += ms; t.rot_launches++; break;
            case ST_GAUGE: t.gauge_ms += ms; t.gauge_launches++; break;
            case ST_BAND: t.bandsum_ms += ms; t.bandsum_launches++; break;
            case ST_RED: t.reduce_ms += ms; t.reduce_launches++; break;
            case ST_RUN: t.run_ms += ms; break;
            default: break;
        }
    }
    t.total_ms = t.ft_ms + t.phase_ms + t.fth_ms + t.eig_ms + t.refine_ms + t.rot_ms + t.gauge_ms + t.bandsum_ms +
                 t.reduce_ms;
    t.h2d_bytes = ctx->h2d;
    t.d2h_bytes = ctx->d2h;
    t.plan_ms = ctx->plan_ms;
    ctx->timing = t;
    return 0;
}

// k-points per chunk: the per-k buffers within 8 GB (3 GB for the FP64 form),
// or within mem_budget / 2 when the context has a budget.
int64_t default_chunk(int N, int nb, bool fp64, size_t mem_budget = 0) {
    size_t per = fp64 ? per_k_bytes<double>(N, nb) : per_k_bytes<float>(N, nb);
    size_t budget = fp64 ? ((size_t)3 << 30) : ((size_t)8 << 30);
    if (mem_budget) budget = std::min(budget, mem_budget / 2);
    int64_t c = (int64_t)(budget / per);
    c = std::min<int64_t>(c, fp64 ? 16384 : 65536);
    c = std::max<int64_t>(64, c & ~(int64_t)63);
    return c;
}

// out[j] = first index of a qx-outermost k list whose qx >= j * nqx (j = 0 ..
// n_slabs), out[n_slabs] = count
void slab_ranges(const int64_t* L, int64_t count, int mp0, int nqx, std::vector<int64_t>& out) {
    const int nslab = (mp0 + nqx - 1) / nqx;
    out.assign(nslab + 1, count);
    int j = 0;
    for (int64_t i = 0; i < count && j < nslab; ++i)
        while (j < nslab && (int)(L[i] % mp0) >= j * nqx) out[j++] = i;
}

// Separable sums for this run when the model, mesh and memory allow them:
// builds (or reuses) the slabs and the (qx, qy)-column ordered k list.
int prepare_sep(mepi_ctx* ctx, const mepi_job* job, int64_t count, bool fp64) {
    ctx->sep_active = false;
    ctx->plan_ms = 0.0;
    if (ctx->ft_pref != 0 || count <= 0) return 0;
    const int mp[3] = {job->mp_grid[0], job->mp_grid[1], job->mp_grid[2]};
    const size_t budget = ctx->mem_budget / 2;   // 0: half the free memory
    const bool reuse = ctx->sep.ready && ctx->sep.fp64 == fp64 && ctx->sep.mp[0] == mp[0] && ctx->sep.mp[1] == mp[1] &&
                       ctx->sep.mp[2] == mp[2] && (budget == 0 || ctx->sep.dev_bytes <= budget);
    if (!reuse) {
        const auto t0 = std::chrono::steady_clock::now();
        sep_plan_free(ctx->sep);
        int rc = sep_plan_build(ctx->sep, ctx->dm, ctx->R_host.data(), ctx->S_host.data(), mp, fp64, budget,
                                ctx->stream);
        if (rc == 1) return 0;
        if (rc) {
            cudaGetLastError();
            return rc;
        }
        ctx->h2d += ctx->sep.h2d_bytes;
        ctx->plan_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    const int64_t key[6] = {mp[0], mp[1], mp[2], job->k_begin, job->k_stride, count};
    if (job->k_list || !std::equal(key, key + 6, ctx->kcol_key)) {
        std::vector<int64_t> L;
        L.reserve(count);
        const int64_t M = (int64_t)mp[0] * mp[1];
        if (job->k_list) {
            // the caller's list, sorted into column order (positions kept for the per-k output)
            auto col = [&](int64_t ki) {
                const int64_t qx = ki % mp[0], qy = (ki / mp[0]) % mp[1], qz = ki / M;
                return (qx * mp[1] + qy) * mp[2] + qz;
            };
            std::vector<int64_t> ord(count);
            for (int64_t i = 0; i < count; ++i) ord[i] = i;
            std::stable_sort(ord.begin(), ord.end(),
                             [&](int64_t a, int64_t b) { return col(job->k_list[a]) < col(job->k_list[b]); });
            for (int64_t i = 0; i < count; ++i) L.push_back(job->k_list[ord[i]]);
            ctx->kpos_host.swap(ord);
        } else {
            for (int qx = 0; qx < mp[0]; ++qx)
                for (int qy = 0; qy < mp[1]; ++qy)
                    for (int qz = 0; qz < mp[2]; ++qz) {
                        const int64_t d = qx + (int64_t)mp[0] * qy + M * qz - job->k_begin;
                        if (d >= 0 && d % job->k_stride == 0 && d / job->k_stride < count)
                            L.push_back(d + job->k_begin);
                    }
            ctx->kpos_host.resize(L.size());
            for (size_t i = 0; i < L.size(); ++i) ctx->kpos_host[i] = (L[i] - job->k_begin) / job->k_stride;
        }
        if ((int64_t)L.size() != count) return MEPI_ERR_ARG;
        CKM(ctx->kcol.ensure(L.size() * sizeof(int64_t)));
        CK(cudaMemcpyAsync(ctx->kcol.p, L.data(), L.size() * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->h2d += L.size() * sizeof(int64_t);
        CKM(ctx->kpos.ensure(std::max<int64_t>(count, 1) * sizeof(int64_t)));
        CK(cudaMemcpyAsync(ctx->kpos.p, ctx->kpos_host.data(), count * sizeof(int64_t), cudaMemcpyHostToDevice,
                           ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->kcol_host.swap(L);
        std::copy(key, key + 6, ctx->kcol_key);
        if (job->k_list) std::fill(ctx->kcol_key, ctx->kcol_key + 6, -1);   // a list is never reused
        ctx->kslab.clear();
    }
    // the list runs qx-outermost: each slab of nqx consecutive qx is one range of it
    if ((int)ctx->kslab.size() < 2 || ctx->kslab_nqx != ctx->sep.nqx) {
        slab_ranges(ctx->kcol_host.data(), count, mp[0], ctx->sep.nqx, ctx->kslab);
        ctx->kslab_nqx = ctx->sep.nqx;
    }
    ctx->sep_active = true;
    return 0;
}

// Phase 1 of a run: validate, size and allocate, build the separable slabs and
// the k list, upload the Fermi and photon energies.  Enqueues only small
// copies and memsets on the context's stream.
int run_prepare(mepi_ctx* ctx, const mepi_job* job, const mepi_acc* out) {
    const int N = ctx->N;
    const int64_t nk_tot = (int64_t)job->mp_grid[0] * job->mp_grid[1] * job->mp_grid[2];
    if (job->mp_grid[0] <= 0 || job->mp_grid[1] <= 0 || job->mp_grid[2] <= 0) return MEPI_ERR_ARG;
    if (job->k_stride <= 0 || job->k_begin < 0) return MEPI_ERR_ARG;
    if (job->n_eF <= 0 || !job->ef_lst || job->valence_bands < 0 || job->valence_bands > N) return MEPI_ERR_ARG;
    if (job->precision != MEPI_PREC_FP64 && job->precision != MEPI_PREC_MIXED) return MEPI_ERR_ARG;
    if (!finite_all(job->ef_lst, job->n_eF) || !std::isfinite(job->T_kelvin)) return MEPI_ERR_ARG;
    const bool opt_hall = (job->outputs & MEPI_OUT_OPT_HALL) != 0;
    if (opt_hall && (job->n_hw <= 0 || !job->hw_lst || !finite_all(job->hw_lst, job->n_hw) ||
                     !std::isfinite(job->eta_smr)))
        return MEPI_ERR_ARG;
    mepi_ctx::Run& r = ctx->run;
    r.job = *job;
    if (job->k_list) {
        if (job->k_count < 0) return MEPI_ERR_ARG;
        for (int64_t i = 0; i < job->k_count; ++i)
            if (job->k_list[i] < 0 || job->k_list[i] >= nk_tot) return MEPI_ERR_ARG;
        r.count = job->k_count;
    } else {
        const int64_t owned =
            job->k_begin < nk_tot ? (nk_tot - job->k_begin + job->k_stride - 1) / job->k_stride : 0;
        r.count = job->k_count < 0 ? owned : std::min<int64_t>(job->k_count, owned);
    }
    r.perk = out && out->perk;
    r.fp64 = job->precision == MEPI_PREC_FP64;
    // an explicit chunk wins; a tuned one is held to the memory budget.  Without a
    // budget the chunk buffers take at most 40% of the memory free now (buffers
    // this context already holds count as free: they are replaced).
    size_t cbudget = ctx->mem_budget;
    if (!cbudget) {
        size_t free_b = 0, total_b = 0;
        CK(cudaMemGetInfo(&free_b, &total_b));
        size_t held = 0;
        for (const DevBuf* d : {&ctx->W, &ctx->E, &ctx->E64, &ctx->H64, &ctx->U, &ctx->Ulo, &ctx->HA, &ctx->OD, &ctx->V,
                                &ctx->CSV, &ctx->flags})
            held += d->bytes;
        cbudget = (size_t)(0.8 * (double)(free_b + held));   // halved inside default_chunk
    }
    const int64_t dchunk = default_chunk(N, ctx->nb, r.fp64, cbudget);
    int64_t chunk = job->chunk_k > 0       ? job->chunk_k
                    : ctx->tune.chunk_k > 0 ? std::min(ctx->tune.chunk_k, ctx->mem_budget ? dchunk : ctx->tune.chunk_k)
                                            : dchunk;
    r.chunk = std::max<int64_t>(1, std::min<int64_t>(chunk, std::max<int64_t>(r.count, 1)));
    r.degen_gap = job->degen_gap >= 0 ? job->degen_gap : 3e-3;
    r.n_hw = opt_hall ? job->n_hw : 0;
    r.L = AccLayout{job->n_eF, job->valence_bands, r.n_hw};
    r.n_cta = bandsum_ctas();
    const AccLayout& L = r.L;
    CKM(ctx->partials.ensure((size_t)r.n_cta * L.size() * sizeof(double)));
    CKM(ctx->out.ensure((size_t)L.size() * sizeof(double) + (size_t)(job->n_eF + r.n_hw) * sizeof(double)));
    CKM(ctx->counters.ensure(4 * sizeof(int)));
    CK(cudaMemsetAsync(ctx->partials.p, 0, (size_t)r.n_cta * L.size() * sizeof(double), ctx->stream));
    CK(cudaMemsetAsync(ctx->counters.p, 0, 4 * sizeof(int), ctx->stream));
    ctx->ev_used = 0;
    if (int r0 = stage_begin(ctx, ST_RUN, &r.run_ev)) return r0;
    double* d_ef = ctx->out.as<double>() + L.size();
    CK(cudaMemcpyAsync(d_ef, job->ef_lst, job->n_eF * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    ctx->h2d += job->n_eF * sizeof(double);
    double* d_hw = d_ef + job->n_eF;
    if (r.n_hw) {
        CK(cudaMemcpyAsync(d_hw, job->hw_lst, r.n_hw * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        ctx->h2d += r.n_hw * sizeof(double);
    }
    JobDev& jb = r.jb;
    jb = JobDev{};
    jb.nE = job->n_eF;
    jb.nval = job->valence_bands;
    jb.do_ahc = (job->outputs & MEPI_OUT_AHC) ? 1 : 0;
    jb.do_mep = (job->outputs & MEPI_OUT_MEP_NIU) ? 1 : 0;
    jb.do_kubo = (job->outputs & MEPI_OUT_KUBO_MEP) ? 1 : 0;
    jb.T_kelvin = job->T_kelvin;
    jb.ef = d_ef;
    jb.nW = r.n_hw;
    jb.hw = r.n_hw ? d_hw : nullptr;
    jb.eta = job->eta_smr;
    if (job->k_list && r.count > 0) {
        CKM(ctx->jlist.ensure(r.count * sizeof(int64_t)));
        CK(cudaMemcpyAsync(ctx->jlist.p, job->k_list, r.count * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
        ctx->h2d += r.count * sizeof(int64_t);
    }
    if (r.perk) CKM(ctx->perk.ensure(std::max<int64_t>(r.count, 1) * 4 * sizeof(double)));
    int rc = prepare_sep(ctx, job, r.count, r.fp64);
    if (rc) return rc;
    rc = r.fp64 ? ensure_chunk<double>(ctx, r.chunk) : ensure_chunk<float>(ctx, r.chunk);
    if (rc) return rc;
    if (!r.fp64) {
        if ((size_t)r.count > ctx->h_flags_cap) {
            if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
            ctx->h_flags = nullptr;
            ctx->h_flags_cap = 0;
            CKM(cudaMallocHost(&ctx->h_flags, std::max<int64_t>(r.count, 1) * sizeof(int)));
            ctx->h_flags_cap = r.count;
        }
        if (!ctx->sep_active && ctx->ft_pref != 2) {
            // the tensor-core operands, allocated here so that the enqueue phase allocates nothing
            if (!ctx->tc.ready()) {
                rc = tc_plan_init(ctx->tc, ctx->dm, ctx->S_host.data());
                if (rc) return rc;
                ctx->h2d += 2 * (int64_t)ctx->tc.ncolp * ctx->tc.Kp * sizeof(__half);
            }
            rc = tc_plan_rows(ctx->tc, r.chunk);
            if (rc) return rc;
        }
    }
    return 0;
}

// chunk c0..c0+cn of the run's k-points: the column-ordered list, or the rank's stride
KRange chunk_range(const mepi_ctx* ctx, int64_t c0, int64_t cn) {
    const mepi_job& job = ctx->run.job;
    if (ctx->sep_active)
        return KRange{0, 1, cn, const_cast<mepi_ctx*>(ctx)->kcol.as<int64_t>() + c0, nullptr,
                      {job.mp_grid[0], job.mp_grid[1], job.mp_grid[2]}};
    if (job.k_list)
        return KRange{0, 1, cn, const_cast<mepi_ctx*>(ctx)->jlist.as<int64_t>() + c0, nullptr,
                      {job.mp_grid[0], job.mp_grid[1], job.mp_grid[2]}};
    return KRange{job.k_begin + c0 * job.k_stride, job.k_stride, cn, nullptr, nullptr,
                  {job.mp_grid[0], job.mp_grid[1], job.mp_grid[2]}};
}

int enqueue_range(mepi_ctx* ctx, int64_t b, int64_t e);

// per-k AHC integrand and gap of the chunk just run (its energies and velocities
// are still in the chunk buffers)
template <typename T>
int enqueue_perk(mepi_ctx* ctx, int64_t cn, const int64_t* pos, int64_t pos0) {
    const mepi_ctx::Run& r = ctx->run;
    STAGE(ST_BAND, launch_perk<T>(ctx->N, cn, ctx->E64.as<double>(), ctx->V.as<cplx<T>>(), r.job.ef_lst[0],
                                  r.job.T_kelvin, pos, pos0, ctx->perk.as<double>(), ctx->stream));
    return 0;
}

// Phase 2: every chunk of the run, as stream work only (no allocation, no
// synchronisation), so that it can be captured into a CUDA graph.
int run_enqueue(mepi_ctx* ctx) {
    mepi_ctx::Run& r = ctx->run;
    if (ctx->sep_active && !ctx->sep.whole()) {
        // one qx slab after the other: build its sums, then run its chunks
        for (size_t j = 0; j + 1 < ctx->kslab.size(); ++j) {
            const int64_t s0 = ctx->kslab[j], s1 = ctx->kslab[j + 1];
            if (s1 <= s0) continue;
            const int qx0 = (int)j * ctx->sep.nqx;
            if (ctx->sep.built_qx0 != qx0) STAGE(ST_FT, launch_sep_slab(ctx->sep, qx0, ctx->stream));
            if (int rc = enqueue_range(ctx, s0, s1)) return rc;
        }
        return 0;
    }
    return enqueue_range(ctx, 0, r.count);
}

// the chunks of run k-points [b, e)
int enqueue_range(mepi_ctx* ctx, int64_t b, int64_t e) {
    mepi_ctx::Run& r = ctx->run;
    int rc = 0;
    for (int64_t c0 = b; c0 < e; c0 += r.chunk) {
        const int64_t cn = std::min(r.chunk, e - c0);
        const KRange kr = chunk_range(ctx, c0, cn);
        // job positions of the chunk's k-points for the per-k output
        const int64_t* pos = ctx->sep_active ? ctx->kpos.as<int64_t>() + c0 : nullptr;
        if (r.fp64) {
            rc = run_chunk<double>(ctx, kr, &r.jb, r.n_cta, 0.0, false, true, nullptr);
            if (!rc && r.perk) rc = enqueue_perk<double>(ctx, cn, pos, c0);
        } else {
            rc = run_chunk<float>(ctx, kr, &r.jb, r.n_cta, r.degen_gap, true, true, nullptr);
            if (!rc && r.perk) rc = enqueue_perk<float>(ctx, cn, pos, c0);
            if (!rc) {
                CK(cudaMemcpyAsync(ctx->h_flags + c0, ctx->flags.p, cn * sizeof(int), cudaMemcpyDeviceToHost,
                                   ctx->stream));
                ctx->d2h += cn * sizeof(int);
            }
        }
        if (rc) return rc;
    }
    return 0;
}

// Phase 3: the FP64 reruns of the mixed form, the fixed-order reduction and
// the copy back.  3a (finish_prepare) reads the rerun flags and makes every
// allocation and plan the reruns need; 3b (finish_launch) enqueues the
// reruns, the reduction and the asynchronous copy back into pinned memory;
// 3c (finish_collect) waits and hands out the results.  The batched form runs
// 3a for every context, then 3b for every context (no allocation there, so no
// implicit device-wide synchronisation: the contexts' reruns overlap on the
// GPU), then 3c.
int finish_prepare(mepi_ctx* ctx) {
    mepi_ctx::Run& r = ctx->run;
    const mepi_job& job = r.job;
    r.redo.clear();
    r.redo_pos.clear();
    r.rslab.clear();
    r.sep_keep = ctx->sep_active;
    if (!r.fp64) {
        CK(cudaStreamSynchronize(ctx->stream));
        for (int64_t i = 0; i < r.count; ++i)
            if (ctx->h_flags[i]) {
                r.redo.push_back(ctx->sep_active ? ctx->kcol_host[i]
                                 : job.k_list    ? job.k_list[i]
                                                 : job.k_begin + i * job.k_stride);
                r.redo_pos.push_back(ctx->sep_active ? ctx->kpos_host[i] : i);
            }
        // A slabbed mixed plan holds FP32 slabs of one qx range: the reruns get
        // FP64 slabs of every block instead, built over their own qx ranges
        // (the reruns are in column order, qx-outermost); the next run rebuilds
        // its plan.  Where no FP64 slab fits, the reruns take the direct sums.
        if (!r.redo.empty() && ctx->sep_active && !ctx->sep.whole()) {
            const int mp[3] = {job.mp_grid[0], job.mp_grid[1], job.mp_grid[2]};
            sep_plan_free(ctx->sep);
            const int prc = sep_plan_build(ctx->sep, ctx->dm, ctx->R_host.data(), ctx->S_host.data(), mp, true,
                                           ctx->mem_budget / 2, ctx->stream);
            if (prc > 1) {
                cudaGetLastError();
                return prc;
            }
            if (prc == 0) ctx->h2d += ctx->sep.h2d_bytes;
            if (prc == 0 && !ctx->sep.whole())
                slab_ranges(r.redo.data(), (int64_t)r.redo.size(), mp[0], ctx->sep.nqx, r.rslab);
        }
        if (!r.redo.empty()) {
            r.rchunk = std::min<int64_t>(default_chunk(ctx->N, ctx->nb, true, ctx->mem_budget), (int64_t)r.redo.size());
            if (int rc = ensure_chunk<double>(ctx, r.rchunk)) return rc;
            CKM(ctx->klist.ensure(r.redo.size() * sizeof(int64_t)));
            CK(cudaMemcpyAsync(ctx->klist.p, r.redo.data(), r.redo.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                               ctx->stream));
            ctx->h2d += r.redo.size() * sizeof(int64_t);
            if (r.perk) {
                CKM(ctx->rpos.ensure(r.redo_pos.size() * sizeof(int64_t)));
                CK(cudaMemcpyAsync(ctx->rpos.p, r.redo_pos.data(), r.redo_pos.size() * sizeof(int64_t),
                                   cudaMemcpyHostToDevice, ctx->stream));
            }
        }
    }
    r.n_redo = (int64_t)r.redo.size();
    const size_t need = r.L.size() + 2;   // the sums, then 4 ints of counters
    if (need > ctx->h_out_cap) {
        if (ctx->h_out) cudaFreeHost(ctx->h_out);
        ctx->h_out = nullptr;
        ctx->h_out_cap = 0;
        CKM(cudaMallocHost(&ctx->h_out, need * sizeof(double)));
        ctx->h_out_cap = need;
    }
    return 0;
}

int finish_launch(mepi_ctx* ctx) {
    mepi_ctx::Run& r = ctx->run;
    const mepi_job& job = r.job;
    const AccLayout& L = r.L;
    int rc = 0;
    if (!r.redo.empty()) {
        if (!ctx->sep.ready || (!ctx->sep.whole() && r.rslab.empty())) ctx->sep_active = false;
        if (r.rslab.empty()) r.rslab = {0, (int64_t)r.redo.size()};
        r.in_reruns = true;
        for (size_t j = 0; j + 1 < r.rslab.size(); ++j) {
            const int64_t b = r.rslab[j], e = r.rslab[j + 1];
            if (e <= b) continue;
            if (ctx->sep_active && !ctx->sep.whole())
                STAGE(ST_FT, launch_sep_slab(ctx->sep, (int)j * ctx->sep.nqx, ctx->stream));
            for (int64_t c0 = b; c0 < e; c0 += r.rchunk) {
                KRange kr{0, 1, std::min<int64_t>(r.rchunk, e - c0), ctx->klist.as<int64_t>() + c0, nullptr,
                          {job.mp_grid[0], job.mp_grid[1], job.mp_grid[2]}};
                rc = run_chunk<double>(ctx, kr, &r.jb, r.n_cta, 0.0, false, true, nullptr);
                if (!rc && r.perk) rc = enqueue_perk<double>(ctx, kr.count, ctx->rpos.as<int64_t>() + c0, 0);
                if (rc) {
                    r.in_reruns = false;
                    return rc;
                }
            }
        }
        r.in_reruns = false;
        ctx->sep_active = r.sep_keep;
    }
    STAGE(ST_RED, launch_reduce(ctx->partials.as<double>(), r.n_cta, L.size(), ctx->out.as<double>(), ctx->stream));
    CK(cudaMemcpyAsync(ctx->h_out, ctx->out.p, L.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(ctx->h_out + L.size(), ctx->counters.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->d2h += L.size() * sizeof(double) + 4 * sizeof(int);
    if (int r1 = stage_end(ctx, r.run_ev)) return r1;
    return 0;
}

// Phase 3c: wait for the context's stream and hand out the results.
int finish_collect(mepi_ctx* ctx, mepi_acc* out) {
    mepi_ctx::Run& r = ctx->run;
    const mepi_job& job = r.job;
    const AccLayout& L = r.L;
    int rc = 0;
    CK(cudaStreamSynchronize(ctx->stream));
    if (r.perk && r.count > 0) {
        CK(cudaMemcpy(out->perk, ctx->perk.p, r.count * 4 * sizeof(double), cudaMemcpyDeviceToHost));
        ctx->d2h += r.count * 4 * sizeof(double);
    }
    const double* h = ctx->h_out;
    int hc[4];
    std::memcpy(hc, h + L.size(), sizeof(hc));
    CK(cudaGetLastError());
    if (ctx->tc.err) {
        int terr = 0;
        CK(cudaMemcpy(&terr, ctx->tc.err, sizeof(int), cudaMemcpyDeviceToHost));
        if (terr) return MEPI_ERR_CUDA;
    }
    rc = collect_timing(ctx, r.count);
    if (rc) return rc;
    const int nE = job.n_eF, nv = job.valence_bands;
    auto put = [&](double* dst, int off, int n) {
        if (dst) std::memcpy(dst, h + off, n * sizeof(double));
    };
    put(out->Ne_sum, L.ne_off(), nE);
    put(out->ahc, L.ahc_off(), 9 * nE);
    put(out->kubo_mep_ic, L.kic_off(), 9 * nE);
    put(out->kubo_mep_lc, L.klc_off(), 9 * nE);
    put(out->kubo_mep_cs, L.kcs_off(), 9 * nE);
    put(out->mep_ic, L.mic_off(), 9 * nv);
    put(out->mep_lc, L.mlc_off(), 9 * nv);
    put(out->mep_cs, L.mcs_off(), 9 * nv);
    if (r.n_hw) {
        put(out->velo_ahc, L.vah_off(), 18 * r.n_hw * nE);
        put(out->kubo_ohc, L.koh_off(), 18 * r.n_hw * nE);
    }
    out->n_k_done = r.count;
    out->n_k_fp64 = r.fp64 ? r.count : r.n_redo;
    out->eig_max_sweeps = hc[0];
    // counters[1] counts FP64 Jacobi launches that hit the sweep cap (an error);
    // FP32 cap hits (counters[2]) were flagged and rerun in FP64; counters[3]
    // is raised by a tensor-core rotation whose bounded wait timed out.
    if (hc[3] != 0) return MEPI_ERR_CUDA;
    if (hc[1] > 0) return MEPI_ERR_EIG;
    return MEPI_OK;
}

int run_impl(mepi_ctx* ctx, const mepi_job* job, mepi_acc* out) {
    int rc = run_prepare(ctx, job, out);
    if (!rc) rc = run_enqueue(ctx);
    if (!rc) rc = finish_prepare(ctx);
    if (!rc) rc = finish_launch(ctx);
    if (!rc) rc = finish_collect(ctx, out);
    return rc;
}

// Device-memory budgets of a batch: each context wants its whole-mesh slabs
// plus its default chunk buffers (x2: the budget is split in halves); the
// total is shared by water-filling, so small models get all they want and the
// large ones split the rest (their slabs are then built per qx range).
std::vector<size_t> batch_budgets(int n, mepi_ctx* const* ctxs, const mepi_job* jobs, double total) {
    std::vector<double> want(n);
    for (int i = 0; i < n; ++i) {
        const bool fp64 = jobs[i].precision == MEPI_PREC_FP64;
        const mepi_ctx* c = ctxs[i];
        const size_t chunk = (size_t)default_chunk(c->N, c->nb, fp64) *
                             (fp64 ? per_k_bytes<double>(c->N, c->nb) : per_k_bytes<float>(c->N, c->nb));
        want[i] = 2.0 * (double)std::max(sep_plan_want(c->dm, c->R_host.data(), jobs[i].mp_grid, fp64), chunk);
        if (c->mem_limit) want[i] = std::min(want[i], (double)c->mem_limit);
    }
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](int a, int b) { return want[a] < want[b]; });
    std::vector<size_t> out(n);
    double left = total;
    for (int j = 0; j < n; ++j) {
        const int i = ord[j];
        const double fair = left / (n - j);
        const double b = std::min(want[i], fair);
        out[i] = (size_t)b;
        left -= b;
    }
    return out;
}

// Process-wide record of tuned launch shapes, keyed by (device, N, nR, blocks).
std::mutex g_tune_mu;
std::map<std::array<int, 4>, mepi_tuning> g_tune;

std::array<int, 4> tune_key(const mepi_ctx* c) { return {c->device, c->N, c->nR, c->nb}; }

}  // namespace

extern "C" {

const char* mepi_version(void) { return "mepinterp-gb300 0.1 (sm_103a)"; }

const char* mepi_strerror(int s) {
    switch (s) {
        case MEPI_OK: return "ok";
        case MEPI_ERR_ARG: return "invalid argument (shape, pointer or option)";
        case MEPI_ERR_CUDA: return "CUDA error or no usable GPU";
        case MEPI_ERR_NOMEM: return "device memory allocation failed";
        case MEPI_ERR_EIG: return "Jacobi eigensolver reached its sweep limit";
        case MEPI_ERR_NONHERM: return "H(R) is not Hermitian (H(-R) != H(R)^dag or -R missing)";
        case MEPI_ERR_NONFINITE: return "NaN or Inf in the model";
        case MEPI_ERR_SCRATCH: return "problem larger than the fixed scratch array of mepi_bandsum_noalloc";
        default: return "unknown status";
    }
}

int mepi_create(mepi_ctx** out, const mepi_model* m) {
    if (!out || !m) return MEPI_ERR_ARG;
    *out = nullptr;
    if (m->n_wf <= 0 || m->n_wf > kMaxN || m->n_R <= 0 || !m->R_frac || !m->H) return MEPI_ERR_ARG;
    if (m->semantics != MEPI_SEM_REF && m->semantics != MEPI_SEM_PAPER) return MEPI_ERR_ARG;
    if (!(m->kubo_tol >= 0.0)) return MEPI_ERR_ARG;
    const int N = m->n_wf, nR = m->n_R;
    const size_t NN = (size_t)N * N;
    if (!finite_all(m->R_frac, 3 * (size_t)nR) || !finite_all(m->H, 2 * NN * nR) || !finite_all(m->a_latt, 9))
        return MEPI_ERR_NONFINITE;
    if (m->r && !finite_all(m->r, 6 * NN * nR)) return MEPI_ERR_NONFINITE;
    if (m->wf_centers && !finite_all(m->wf_centers, 3 * (size_t)N)) return MEPI_ERR_NONFINITE;
    // Hermiticity: H(n,m,-R) = conj(H(m,n,R))
    double hmax = 0;
    for (size_t i = 0; i < 2 * NN * nR; ++i) hmax = std::max(hmax, std::fabs(m->H[i]));
    const double htol = 1e-6 * hmax + 1e-9;
    for (int r = 0; r < nR; ++r) {
        int rm = -1;
        for (int s = 0; s < nR && rm < 0; ++s) {
            bool eq = true;
            for (int i = 0; i < 3; ++i) eq = eq && std::fabs(m->R_frac[3 * s + i] + m->R_frac[3 * r + i]) <= 1e-9;
            if (eq) rm = s;
        }
        if (rm < 0) return MEPI_ERR_NONHERM;
        for (int a = 0; a < N; ++a)
            for (int b = 0; b < N; ++b) {
                const double* x = m->H + 2 * (a + N * b + NN * r);
                const double* y = m->H + 2 * (b + N * a + NN * rm);
                if (std::fabs(x[0] - y[0]) > htol || std::fabs(x[1] + y[1]) > htol) return MEPI_ERR_NONHERM;
            }
    }
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count <= 0) {
        cudaGetLastError();
        return MEPI_ERR_CUDA;
    }
    mepi_ctx* ctx = new (std::nothrow) mepi_ctx();
    if (!ctx) return MEPI_ERR_NOMEM;
    auto fail = [&](int code) {
        mepi_destroy(ctx);
        return code;
    };
    if (cudaGetDevice(&ctx->device) != cudaSuccess) return fail(MEPI_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(MEPI_ERR_CUDA);
    ctx->N = N;
    ctx->nR = nR;
    ctx->nb = m->r ? 10 : 4;
    std::memcpy(ctx->a_latt, m->a_latt, sizeof(ctx->a_latt));
    // derivative weights: dR_cart = matmul(a_latt, dR) or 2 pi dR
    double C[9];
    for (int a = 0; a < 3; ++a)
        for (int j = 0; j < 3; ++j) C[a * 3 + j] = m->use_cart_velo ? m->a_latt[a + 3 * j] : (a == j ? 2.0 * kPi : 0.0);
    // Fourier stack
    const int nb = ctx->nb;
    std::vector<cplx<double>> S;
    try {
        S.resize((size_t)nR * NN * nb);
    } catch (...) {
        return fail(MEPI_ERR_NOMEM);
    }
    const int qa[3] = {0, 0, 1}, qb[3] = {1, 2, 2};
    for (int r = 0; r < nR; ++r) {
        double CR[3];
        for (int a = 0; a < 3; ++a)
            CR[a] = C[a * 3 + 0] * m->R_frac[3 * r] + C[a * 3 + 1] * m->R_frac[3 * r + 1] + C[a * 3 + 2] * m->R_frac[3 * r + 2];
        for (int n = 0; n < N; ++n)
            for (int mm = 0; mm < N; ++mm) {
                cplx<double>* s = &S[((size_t)r * NN + n * N + mm) * nb];
                const double* h = m->H + 2 * (n + (size_t)N * mm + NN * r);
                cplx<double> H = mk(h[0], h[1]);
                s[0] = H;
                for (int a = 0; a < 3; ++a) s[1 + a] = CR[a] * H;
                if (m->r) {
                    cplx<double> rv[3];
                    for (int b = 0; b < 3; ++b) {
                        const double* x = m->r + 2 * (b + 3 * (n + (size_t)N * (mm + (size_t)N * r)));
                        rv[b] = mk(x[0], x[1]);
                        s[4 + b] = rv[b];
                    }
                    for (int q = 0; q < 3; ++q) s[7 + q] = CR[qa[q]] * rv[qb[q]] - CR[qb[q]] * rv[qa[q]];
                }
            }
    }
    // MEPI_FT=tc or =simt forces the tensor-core or SIMT Fourier sums (tests of
    // the non-separable paths); the default takes the separable sums when the
    // model and mesh allow them
    const char* ft_env = std::getenv("MEPI_FT");
    ctx->ft_pref = (ft_env && std::strcmp(ft_env, "tc") == 0) ? 1 : (ft_env && std::strcmp(ft_env, "simt") == 0) ? 2 : 0;
    // MEPI_ROT=simt forces the CUDA-core rotation in the mixed form (comparisons)
    const char* rot_env = std::getenv("MEPI_ROT");
    ctx->rot_pref = (rot_env && std::strcmp(rot_env, "simt") == 0) ? 2 : 0;
    // MEPI_JACOBI_THETA overrides the FP32 Jacobi's gap-relative stop (0 = run to the FP32 floor)
    if (const char* th = std::getenv("MEPI_JACOBI_THETA")) ctx->jacobi_theta = (float)std::atof(th);
    if (const char* jf = std::getenv("MEPI_JACOBI"))
        ctx->jacobi_warp = std::strcmp(jf, "smem") == 0 ? 0 : (std::strcmp(jf, "warp3") == 0 ? 2 : 1);
    std::vector<double> Rh(3 * (size_t)nR);
    std::memcpy(Rh.data(), m->R_frac, Rh.size() * sizeof(double));
    if (ctx->S.ensure(S.size() * sizeof(cplx<double>)) != cudaSuccess) return fail(MEPI_ERR_NOMEM);
    if (ctx->R.ensure(Rh.size() * sizeof(double)) != cudaSuccess) return fail(MEPI_ERR_NOMEM);
    if (cudaMemcpy(ctx->S.p, S.data(), S.size() * sizeof(cplx<double>), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(MEPI_ERR_CUDA);
    ctx->h2d += S.size() * sizeof(cplx<double>) + Rh.size() * sizeof(double);
    ctx->S_host.swap(S);
    ctx->R_host = Rh;
    if (cudaMemcpy(ctx->R.p, Rh.data(), Rh.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(MEPI_ERR_CUDA);
    if (m->wf_centers) {
        if (ctx->tau.ensure(3 * (size_t)N * sizeof(double)) != cudaSuccess) return fail(MEPI_ERR_NOMEM);
        if (cudaMemcpy(ctx->tau.p, m->wf_centers, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(MEPI_ERR_CUDA);
        ctx->h2d += 3 * (size_t)N * sizeof(double);
    }
    DevModel& d = ctx->dm;
    d.N = N;
    d.nR = nR;
    d.nb = nb;
    d.has_r = m->r ? 1 : 0;
    d.has_tau = m->wf_centers ? 1 : 0;
    d.semantics = m->semantics;
    d.do_gauge = m->do_gauge_trafo ? 1 : 0;
    d.kubo_tol = m->kubo_tol;
    std::memcpy(d.C, C, sizeof(C));
    d.S = ctx->S.as<cplx<double>>();
    d.R = ctx->R.as<double>();
    d.tau = m->wf_centers ? ctx->tau.as<double>() : nullptr;
    {
        // launch shapes tuned earlier in this process for the same kind of model
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(tune_key(ctx));
        if (it != g_tune.end()) ctx->tune = it->second;
    }
    *out = ctx;
    return MEPI_OK;
}

int mepi_run(mepi_ctx* ctx, const mepi_job* job, mepi_acc* out) {
    if (!ctx || !job || !out) return MEPI_ERR_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return MEPI_ERR_CUDA;
    try {
        return run_impl(ctx, job, out);
    } catch (const std::bad_alloc&) {
        return MEPI_ERR_NOMEM;
    } catch (...) {
        return MEPI_ERR_CUDA;
    }
}

int mepi_interp_k(mepi_ctx* ctx, int32_t precision, int64_t n_k, const double* kpts, double* en_k, double* V_ka,
                  double* A_diag, double* Om_diag) {
    if (!ctx || n_k < 0 || (n_k > 0 && (!kpts || !en_k || !V_ka))) return MEPI_ERR_ARG;
    if (precision != MEPI_PREC_FP64 && precision != MEPI_PREC_MIXED) return MEPI_ERR_ARG;
    if (n_k == 0) return MEPI_OK;
    if (!finite_all(kpts, 3 * (size_t)n_k)) return MEPI_ERR_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return MEPI_ERR_CUDA;
    try {
        const int N = ctx->N;
        const size_t NN = (size_t)N * N;
        const bool fp64 = precision == MEPI_PREC_FP64;
        const int64_t chunk = std::min<int64_t>(n_k, 4096);
        int rc = fp64 ? ensure_chunk<double>(ctx, chunk) : ensure_chunk<float>(ctx, chunk);
        if (rc) return rc;
        const size_t esz = fp64 ? sizeof(double) : sizeof(float);
        CKM(ctx->ODH.ensure(chunk * 3 * N * 2 * esz));
        CKM(ctx->kpts.ensure(n_k * 3 * sizeof(double)));
        CKM(ctx->counters.ensure(4 * sizeof(int)));
        CK(cudaMemsetAsync(ctx->counters.p, 0, 4 * sizeof(int), ctx->stream));
        CK(cudaMemcpyAsync(ctx->kpts.p, kpts, n_k * 3 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        ctx->ev_used = 0;
        std::vector<double> hE, hV, hHA, hO;
        for (int64_t c0 = 0; c0 < n_k; c0 += chunk) {
            const int64_t cn = std::min(chunk, n_k - c0);
            KRange kr{0, 1, cn, nullptr, ctx->kpts.as<double>() + 3 * c0, {1, 1, 1}};
            if (fp64)
                rc = run_chunk<double>(ctx, kr, nullptr, 0, 0.0, false, false, ctx->ODH.as<cplx<double>>());
            else
                rc = run_chunk<float>(ctx, kr, nullptr, 0, 0.0, false, false, ctx->ODH.as<cplx<float>>());
            if (rc) return rc;
            // copy back and convert to double
            std::vector<unsigned char> bV(cn * 3 * NN * 2 * esz), bHA(cn * 6 * NN * 2 * esz), bO(cn * 3 * N * 2 * esz);
            std::vector<double> bE(cn * N);
            CK(cudaMemcpyAsync(bE.data(), ctx->E64.p, bE.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaMemcpyAsync(bV.data(), ctx->V.p, bV.size(), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaMemcpyAsync(bHA.data(), ctx->HA.p, bHA.size(), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaMemcpyAsync(bO.data(), ctx->ODH.p, bO.size(), cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
            auto conv = [&](const std::vector<unsigned char>& b, std::vector<double>& dst) {
                size_t n = b.size() / esz;
                size_t off = dst.size();
                dst.resize(off + n);
                if (fp64) std::memcpy(dst.data() + off, b.data(), b.size());
                else {
                    const float* f = reinterpret_cast<const float*>(b.data());
                    for (size_t i = 0; i < n; ++i) dst[off + i] = f[i];
                }
            };
            hE.insert(hE.end(), bE.begin(), bE.end());
            conv(bV, hV);
            conv(bHA, hHA);
            conv(bO, hO);
        }
        int hc[4];
        CK(cudaMemcpy(hc, ctx->counters.p, sizeof(hc), cudaMemcpyDeviceToHost));
        if (hc[3] != 0) return MEPI_ERR_CUDA;
        if (ctx->tc.err) {
            int terr = 0;
            CK(cudaMemcpy(&terr, ctx->tc.err, sizeof(int), cudaMemcpyDeviceToHost));
            if (terr) return MEPI_ERR_CUDA;
        }
        // scatter into the Fortran layouts
        for (int64_t k = 0; k < n_k; ++k) {
            for (int n = 0; n < N; ++n) en_k[k * N + n] = hE[k * N + n];
            for (int a = 0; a < 3; ++a)
                for (int n = 0; n < N; ++n)
                    for (int mm = 0; mm < N; ++mm) {
                        size_t src = 2 * (((size_t)k * 3 + a) * NN + n * N + mm);
                        size_t dst = 2 * (a + 3 * (n + (size_t)N * (mm + (size_t)N * k)));
                        V_ka[dst] = hV[src];
                        V_ka[dst + 1] = hV[src + 1];
                    }
            if (A_diag)
                for (int n = 0; n < N; ++n)
                    for (int c = 0; c < 3; ++c) {
                        size_t src = 2 * (((size_t)k * 6 + 3 + c) * NN + n * N + n);
                        size_t dst = 2 * (c + 3 * (n + (size_t)N * k));
                        A_diag[dst] = hHA[src];
                        A_diag[dst + 1] = hHA[src + 1];
                    }
            if (Om_diag) {
                const int qa[3] = {0, 0, 1}, qb[3] = {1, 2, 2};
                for (int n = 0; n < N; ++n) {
                    double om[3][3][2];
                    std::memset(om, 0, sizeof(om));
                    for (int q = 0; q < 3; ++q) {
                        size_t src = 2 * (((size_t)k * 3 + q) * N + n);
                        double re = hO[src], im = hO[src + 1];
                        om[qa[q]][qb[q]][0] = re;
                        om[qa[q]][qb[q]][1] = im;
                        om[qb[q]][qa[q]][0] = -re;
                        om[qb[q]][qa[q]][1] = -im;
                    }
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) {
                            size_t dst = 2 * (a + 3 * (b + 3 * (n + (size_t)N * k)));
                            Om_diag[dst] = om[a][b][0];
                            Om_diag[dst + 1] = om[a][b][1];
                        }
                }
            }
        }
        if (fp64 && hc[1] > 0) return MEPI_ERR_EIG;
        return MEPI_OK;
    } catch (const std::bad_alloc&) {
        return MEPI_ERR_NOMEM;
    } catch (...) {
        return MEPI_ERR_CUDA;
    }
}

int mepi_get_timing(const mepi_ctx* ctx, mepi_timing* t) {
    if (!ctx || !t) return MEPI_ERR_ARG;
    *t = ctx->timing;
    return MEPI_OK;
}

int mepi_set_tuning(mepi_ctx* ctx, const mepi_tuning* t) {
    if (!ctx || !t || t->jacobi_threads < 0 || t->jacobi_kblock < 0 || t->chunk_k < 0) return MEPI_ERR_ARG;
    if (t->jacobi_threads && (t->jacobi_threads % 32 || t->jacobi_threads > 256)) return MEPI_ERR_ARG;
    ctx->tune = *t;
    return MEPI_OK;
}

int mepi_set_mem_limit(mepi_ctx* ctx, uint64_t bytes) {
    if (!ctx) return MEPI_ERR_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return MEPI_ERR_CUDA;
    ctx->mem_limit = ctx->mem_budget = (size_t)bytes;
    if (bytes && run_buffer_bytes(ctx) > bytes) release_run_buffers(ctx);
    return MEPI_OK;
}

int mepi_trim(mepi_ctx* ctx) {
    if (!ctx) return MEPI_ERR_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return MEPI_ERR_CUDA;
    release_run_buffers(ctx);
    return MEPI_OK;
}

int mepi_get_tuning(const mepi_ctx* ctx, mepi_tuning* t) {
    if (!ctx || !t) return MEPI_ERR_ARG;
    *t = ctx->tune;
    return MEPI_OK;
}

int mepi_autotune(mepi_ctx* ctx, const mepi_job* job, int64_t sample_k, mepi_tuning* best) {
    if (!ctx || !job) return MEPI_ERR_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return MEPI_ERR_CUDA;
    try {
        mepi_job j = *job;
        j.k_begin = 0;
        j.k_stride = 1;
        j.k_count = sample_k > 0 ? sample_k : 32768;
        j.chunk_k = 0;
        mepi_acc acc{};
        const mepi_tuning saved = ctx->tune;
        ctx->tune = mepi_tuning{};
        int rc = run_impl(ctx, &j, &acc);   // builds the slabs; also a warm-up
        if (rc) {
            ctx->tune = saved;
            return rc;
        }
        const int np = ctx->N <= 8 ? 8 : ctx->N <= 16 ? 16 : ctx->N <= 32 ? 32 : 64;
        mepi_tuning win{};
        double best_ms = 1e300;
        // chunk candidates: the default (8 GB of per-k buffers, at most 65,536 k) and a quarter of it
        const int64_t c_def = default_chunk(ctx->N, ctx->nb, j.precision == MEPI_PREC_FP64, ctx->mem_limit);
        const int64_t c_q = std::max<int64_t>(64, (c_def / 4) & ~(int64_t)63);
        for (int threads : {64, 128, 256}) {
            if (threads < np / 2) continue;
            for (int kb : {4, 8, 16})
                for (int64_t ch : {c_q, c_def}) {
                    ctx->tune = mepi_tuning{threads, kb, ch, 0.0};
                    rc = run_impl(ctx, &j, &acc);
                    if (rc) {
                        ctx->tune = saved;
                        return rc;
                    }
                    const double ms = ctx->timing.run_ms;
                    if (ms < best_ms) {
                        best_ms = ms;
                        win = ctx->tune;
                        win.k_per_s = (double)acc.n_k_done / (ms * 1e-3);
                    }
                }
        }
        ctx->tune = win;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tune[tune_key(ctx)] = win;
        }
        if (best) *best = win;
        // leave no run buffers behind, so that many contexts can be tuned in turn
        release_run_buffers(ctx);
        return MEPI_OK;
    } catch (const std::bad_alloc&) {
        return MEPI_ERR_NOMEM;
    } catch (...) {
        return MEPI_ERR_CUDA;
    }
}

int mepi_run_batch(int32_t n, mepi_ctx* const* ctxs, const mepi_job* jobs, mepi_acc* accs, double* graph_ms) {
    if (n < 0 || (n > 0 && (!ctxs || !jobs || !accs))) return MEPI_ERR_ARG;
    if (n == 0) return MEPI_OK;
    for (int i = 0; i < n; ++i)
        if (!ctxs[i] || ctxs[i]->device != ctxs[0]->device) return MEPI_ERR_ARG;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j)
            if (ctxs[i] == ctxs[j]) return MEPI_ERR_ARG;   // one run per context
    if (cudaSetDevice(ctxs[0]->device) != cudaSuccess) return MEPI_ERR_CUDA;
    cudaStream_t bs = nullptr;
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    std::vector<cudaEvent_t> join(n, nullptr);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto cleanup = [&](int rc) {
        for (int i = 0; i < n; ++i) {
            ctxs[i]->timed = true;
            ctxs[i]->mem_budget = ctxs[i]->mem_limit;
        }
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (cudaEvent_t e : join)
            if (e) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (t0) cudaEventDestroy(t0);
        if (t1) cudaEventDestroy(t1);
        if (bs) cudaStreamDestroy(bs);
        return rc;
    };
    try {
        // 1. prepare every context (allocations, slabs, k lists), outside the capture;
        //    the contexts share 80% of the device memory free now (their own
        //    slabs and chunk buffers count as free: they are released first)
        size_t free_b = 0, total_b = 0, held = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return cleanup(MEPI_ERR_CUDA);
        for (int i = 0; i < n; ++i) held += run_buffer_bytes(ctxs[i]);
        const std::vector<size_t> budget = batch_budgets(n, ctxs, jobs, (double)(free_b + held) * 0.8);
        for (int i = 0; i < n; ++i)
            if (run_buffer_bytes(ctxs[i]) > budget[i]) release_run_buffers(ctxs[i]);
        for (int i = 0; i < n; ++i) {
            ctxs[i]->timed = false;
            ctxs[i]->mem_budget = budget[i];
            int rc = run_prepare(ctxs[i], &jobs[i], &accs[i]);
            if (rc) return cleanup(rc);
        }
        for (int i = 0; i < n; ++i)
            if (cudaStreamSynchronize(ctxs[i]->stream) != cudaSuccess) return cleanup(MEPI_ERR_CUDA);
        if (cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking) != cudaSuccess) return cleanup(MEPI_ERR_CUDA);
        if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) return cleanup(MEPI_ERR_CUDA);
        for (int i = 0; i < n; ++i)
            if (cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming) != cudaSuccess) return cleanup(MEPI_ERR_CUDA);
        // 2. capture every context's chunk pipeline on its own stream into one graph
        if (cudaStreamBeginCapture(bs, cudaStreamCaptureModeRelaxed) != cudaSuccess) return cleanup(MEPI_ERR_CUDA);
        int rc = cudaEventRecord(fork, bs) == cudaSuccess ? 0 : MEPI_ERR_CUDA;
        for (int i = 0; i < n && !rc; ++i) {
            if (cudaStreamWaitEvent(ctxs[i]->stream, fork, 0) != cudaSuccess) { rc = MEPI_ERR_CUDA; break; }
            rc = run_enqueue(ctxs[i]);
            if (!rc && (cudaEventRecord(join[i], ctxs[i]->stream) != cudaSuccess ||
                        cudaStreamWaitEvent(bs, join[i], 0) != cudaSuccess))
                rc = MEPI_ERR_CUDA;
        }
        const cudaError_t ec = cudaStreamEndCapture(bs, &graph);
        if (rc) return cleanup(rc);
        if (ec != cudaSuccess || !graph) return cleanup(MEPI_ERR_CUDA);
        if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) return cleanup(MEPI_ERR_CUDA);
        // 3. one launch
        if (cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess) return cleanup(MEPI_ERR_CUDA);
        if (cudaEventRecord(t0, bs) != cudaSuccess || cudaGraphLaunch(exec, bs) != cudaSuccess ||
            cudaEventRecord(t1, bs) != cudaSuccess || cudaStreamSynchronize(bs) != cudaSuccess)
            return cleanup(MEPI_ERR_CUDA);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, t0, t1) != cudaSuccess) return cleanup(MEPI_ERR_CUDA);
        if (graph_ms) *graph_ms = ms;
        // 4. reruns, reductions and copies back: every context's allocations
        //    first, then every context's launches (they overlap on the GPU),
        //    then the results
        for (int i = 0; i < n; ++i) {
            rc = finish_prepare(ctxs[i]);
            if (rc) return cleanup(rc);
        }
        for (int i = 0; i < n; ++i) {
            rc = finish_launch(ctxs[i]);
            if (rc) return cleanup(rc);
        }
        for (int i = 0; i < n; ++i) {
            rc = finish_collect(ctxs[i], &accs[i]);
            if (rc) return cleanup(rc);
        }
        return cleanup(MEPI_OK);
    } catch (const std::bad_alloc&) {
        return cleanup(MEPI_ERR_NOMEM);
    } catch (...) {
        return cleanup(MEPI_ERR_CUDA);
    }
}

int mepi_destroy(mepi_ctx* ctx) {
    if (!ctx) return MEPI_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (DevBuf* b : {&ctx->S, &ctx->R, &ctx->tau, &ctx->W, &ctx->E, &ctx->E64, &ctx->H64, &ctx->U, &ctx->Ulo, &ctx->HA,
                      &ctx->OD, &ctx->V, &ctx->CSV,
                      &ctx->ODH, &ctx->flags, &ctx->klist, &ctx->kpts, &ctx->partials, &ctx->out, &ctx->counters,
                      &ctx->jlist, &ctx->kpos, &ctx->rpos, &ctx->perk, &ctx->kcol})
        b->release();
    for (auto& ev : ctx->events) {
        cudaEventDestroy(ev.a);
        cudaEventDestroy(ev.b);
    }
    if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
    if (ctx->h_out) cudaFreeHost(ctx->h_out);
    tc_plan_free(ctx->tc);
    sep_plan_free(ctx->sep);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MEPI_OK;
}

}  // extern "C"
