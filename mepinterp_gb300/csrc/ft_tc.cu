// Tensor-core Fourier sums for the mixed form (tcgen05 + TMA, sm_103a).
//
// The complex GEMM X[k][c] = sum_R exp(2 pi i k.R) S[R][c] of FT_R_to_k
// (src/wann_interp.f90:151-384) is run as one real GEMM
//     C'[k][2c + t] = sum_{kappa} A'[k][kappa] B'[2c + t][kappa]
// with A'[k][2R] = cos(2 pi k.R), A'[k][2R+1] = sin(2 pi k.R) and
// B'[2c][2R] = Re S, B'[2c][2R+1] = -Im S, B'[2c+1][2R] = Im S,
// B'[2c+1][2R+1] = Re S, so C'[k][2c] = Re X and C'[k][2c+1] = Im X.
// Both operands are split into FP16 hi + lo parts (x = hi + lo, lo the FP16
// rounding of the residual) and the product is formed from three tcgen05.mma
// passes hi*hi + hi*lo + lo*hi accumulating in FP32 in tensor memory; lo*lo
// (~2^-22 relative) is dropped.  A' is scaled by 2^12 and each stack block of
// B' by its own power of two so that no lo part underflows into FP16
// subnormals; the epilogue divides the scales out exactly.
//
// Operands are K-major (K contiguous) with a 128-byte swizzle; TMA fills a
// 3-stage shared-memory ring (mbarrier full/empty pairs), one elected thread
// issues the MMAs (M = 128 k-points, N = one column tile, K = 16 per
// instruction), and four epilogue warps read the accumulator with tcgen05.ld
// (warp w reads TMEM lanes 32*(w%4)..+31 = its k rows), apply the
// tight-binding phase epilogue of ft.cu in FP32 and write the W-gauge blocks.
// Column tiles hold PT whole (n,m) pairs x all stack blocks, ordered
// (blk, pair, re/im), so each thread has every block of its pairs.
// Every mbarrier wait is bounded; on a timeout the CTA raises *err and
// skips the rest of its work, still releasing its tensor memory.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mepi_internal.cuh"
#include "ft_tc.cuh"
#include "tc_common.cuh"

namespace mepi {

namespace {

using namespace tc;

constexpr int BM = 128;            // k-points per tile (TMEM lanes)
constexpr int BK = 64;             // K elements per stage (128 B of FP16)
constexpr int STAGES = 3;
constexpr int NTHREADS = 192;      // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
template <int NB>
struct TcEpi {
    int N, NN, PT, nb;
    int has_tau;
    float C[9];
    float inv_scale[NB];
    const double* tau;
    KRange kr;
    cplx<float>* W;
};

// ---------------------------------------------------------------------------
template <int NB, int TN>
__global__ void __launch_bounds__(NTHREADS, 1)
    ft_tc_kernel(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                 const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl, int nkb,
                 TcEpi<NB> ep, int* err) {
    constexpr uint32_t A_BYTES = BM * BK * 2;
    constexpr uint32_t B_BYTES = TN * BK * 2;
    constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
    constexpr uint32_t TMEM_COLS = TN <= 32 ? 32 : TN <= 64 ? 64 : TN <= 128 ? 128 : 256;
    constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* accum = empty + STAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_tile = blockIdx.x, m_tile = blockIdx.y;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    int issued = 0;  // TMA stages issued by the producer (for the abort drain)
    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer ----------------
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % STAGES;
            const uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
            if (*abort_flag) break;
            if (!mbar_wait(&empty[s], ph ^ 1u)) {
                *abort_flag = 1;
                atomicExch(err, 1);
                break;
            }
            unsigned char* st = smem + s * STAGE_BYTES;
            mbar_expect_tx(&full[s], STAGE_BYTES);
            tma_load_2d(st, &tmAh, kb * BK, m_tile * BM, &full[s]);
            tma_load_2d(st + A_BYTES, &tmAl, kb * BK, m_tile * BM, &full[s]);
            tma_load_2d(st + 2 * A_BYTES, &tmBh, kb * BK, n_tile * TN, &full[s]);
            tma_load_2d(st + 2 * A_BYTES + B_BYTES, &tmBl, kb * BK, n_tile * TN, &full[s]);
            ++issued;
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer ----------------
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % STAGES;
            const uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
            if (*abort_flag || !mbar_wait(&full[s], ph)) {
                *abort_flag = 1;
                atomicExch(err, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            unsigned char* st = smem + s * STAGE_BYTES;
            const uint64_t ah = sw128_desc(st), al = sw128_desc(st + A_BYTES);
            const uint64_t bh = sw128_desc(st + 2 * A_BYTES), bl = sw128_desc(st + 2 * A_BYTES + B_BYTES);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk) {
                const uint64_t off = (uint64_t)(kk * 32) >> 4;  // 16 FP16 = 32 bytes along K
                mma_f16(tmem, ah + off, bh + off, IDESC, (kb | kk) != 0 ? 1u : 0u);
                mma_f16(tmem, ah + off, bl + off, IDESC, 1u);
                mma_f16(tmem, al + off, bh + off, IDESC, 1u);
            }
            mma_commit(&empty[s]);
        }
        // always: tracks completion of every MMA issued, also after an abort
        mma_commit(accum);
    } else if (warp >= 2) {
        // ---------------- epilogue ----------------
        const bool ok = mbar_wait(accum, 0);
        if (!ok) {
            *abort_flag = 1;
            atomicExch(err, 1);
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int quad = warp & 3;
        const int row = quad * 32 + lane;
        const int64_t i = (int64_t)m_tile * BM + row;
        const bool valid = ok && (i < ep.kr.count);
        float k[3] = {0.f, 0.f, 0.f};
        if (valid) {
            double kd[3];
            if (ep.kr.kpts) {
                kd[0] = ep.kr.kpts[3 * i]; kd[1] = ep.kr.kpts[3 * i + 1]; kd[2] = ep.kr.kpts[3 * i + 2];
            } else {
                mp_kpt(ep.kr.mp, k_of(ep.kr, i), kd);
            }
            k[0] = (float)kd[0]; k[1] = (float)kd[1]; k[2] = (float)kd[2];
        }
        const uint32_t tbase = tmem + ((uint32_t)(quad * 32) << 16);
        cplx<float>* Wk = ep.W + (size_t)(valid ? i : 0) * NB * ep.NN;
        for (int q4 = 0; q4 < ep.PT / 4; ++q4) {
            float x[NB][8];
#pragma unroll
            for (int b = 0; b < NB; ++b) tmem_ld8(tbase + (uint32_t)(b * 2 * ep.PT + 8 * q4), x[b]);
            tmem_wait_ld();
            if (!valid) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int pair = n_tile * ep.PT + 4 * q4 + j;
                if (pair >= ep.NN) continue;
                const int n = pair / ep.N, m = pair % ep.N;
                cplx<float> X[NB];
#pragma unroll
                for (int b = 0; b < NB; ++b) X[b] = mk(x[b][2 * j] * ep.inv_scale[b], x[b][2 * j + 1] * ep.inv_scale[b]);
                cplx<float> psi = mk(1.f, 0.f);
                float dt[3] = {0.f, 0.f, 0.f};
                if (ep.has_tau) {
                    float d[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) d[c] = (float)(ep.tau[m * 3 + c] - ep.tau[n * 3 + c]);
                    float xx = k[0] * d[0] + k[1] * d[1] + k[2] * d[2];
                    xx -= rintf(xx);  // psi = exp(2 pi i xx) has period 1 in xx
                    float s, c;
                    sincospif(2.f * xx, &s, &c);
                    psi = mk(c, s);
#pragma unroll
                    for (int a = 0; a < 3; ++a) dt[a] = ep.C[a * 3] * d[0] + ep.C[a * 3 + 1] * d[1] + ep.C[a * 3 + 2] * d[2];
                }
                cplx<float> H = psi * X[0];
                Wk[pair] = H;
#pragma unroll
                for (int a = 0; a < 3; ++a) Wk[(size_t)(1 + a) * ep.NN + pair] = times_i(psi * X[1 + a] + dt[a] * H);
                if constexpr (NB == 10) {
                    cplx<float> A[3];
#pragma unroll
                    for (int b = 0; b < 3; ++b) {
                        A[b] = psi * X[4 + b];
                        Wk[(size_t)(4 + b) * ep.NN + pair] = A[b];
                    }
                    Wk[(size_t)7 * ep.NN + pair] = times_i(psi * X[7] + dt[0] * A[1] - dt[1] * A[0]);
                    Wk[(size_t)8 * ep.NN + pair] = times_i(psi * X[8] + dt[0] * A[2] - dt[2] * A[0]);
                    Wk[(size_t)9 * ep.NN + pair] = times_i(psi * X[9] + dt[1] * A[2] - dt[2] * A[1]);
                }
            }
        }
    }
    __syncwarp();
    // On abort, let every TMA copy and MMA this CTA issued finish before shared
    // and tensor memory are released (bounded waits).
    if (warp == 0 && lane == 0 && *abort_flag) {
        for (int kb = issued - STAGES > 0 ? issued - STAGES : 0; kb < issued; ++kb)
            mbar_wait(&full[kb % STAGES], (uint32_t)(kb / STAGES) & 1u);
    }
    if (warp == 1 && lane == 0 && *abort_flag) mbar_wait(accum, 0);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// A' hi/lo for one chunk: rows i < count get cos/sin(2 pi k.R) * 2^12, the
// rest (and K padding) zeros.  The angle 2 k.R is formed in FP64 and reduced
// to [-1, 1] before the FP32 sincospi.
__global__ void phase_split_kernel(KRange kr, const double* __restrict__ R, int nR, int Kp, int rows,
                                   __half2* __restrict__ Ah, __half2* __restrict__ Al) {
    const int halfK = Kp / 2;
    const int64_t total = (int64_t)rows * halfK;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / halfK;
        const int r = (int)(t % halfK);
        float c = 0.f, s = 0.f;
        if (i < kr.count && r < nR) {
            double k[3];
            if (kr.kpts) {
                k[0] = kr.kpts[3 * i]; k[1] = kr.kpts[3 * i + 1]; k[2] = kr.kpts[3 * i + 2];
            } else {
                mp_kpt(kr.mp, k_of(kr, i), k);
            }
            double x = 2.0 * (k[0] * R[3 * r] + k[1] * R[3 * r + 1] + k[2] * R[3 * r + 2]);
            x -= 2.0 * rint(0.5 * x);
            sincospif((float)x, &s, &c);
        }
        const float sc = kTcAScale;
        float vc = c * sc, vs = s * sc;
        __half hc = __float2half_rn(vc), hs = __float2half_rn(vs);
        __half lc = __float2half_rn(vc - __half2float(hc)), ls = __float2half_rn(vs - __half2float(hs));
        Ah[t] = __halves2half2(hc, hs);
        Al[t] = __halves2half2(lc, ls);
    }
}

template <int NB, int TN>
size_t tc_smem_bytes() {
    return (size_t)STAGES * (2 * BM * BK * 2 + 2 * TN * BK * 2) + 1024 + 256;
}

template <int NB, int TN>
cudaError_t launch_tc_t(const TcPlan& p, const KRange& kr, cplx<float>* W, cudaStream_t s) {
    TcEpi<NB> ep;
    ep.N = p.N;
    ep.NN = p.N * p.N;
    ep.PT = p.PT;
    ep.nb = NB;
    ep.has_tau = p.tau != nullptr;
    for (int i = 0; i < 9; ++i) ep.C[i] = (float)p.C[i];
    for (int b = 0; b < NB; ++b) ep.inv_scale[b] = p.inv_scale[b];
    ep.tau = p.tau;
    ep.kr = kr;
    ep.W = W;
    const size_t smem = tc_smem_bytes<NB, TN>();
    cudaError_t e = cudaFuncSetAttribute(ft_tc_kernel<NB, TN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)p.n_tiles, (unsigned)(p.rows / BM));
    ft_tc_kernel<NB, TN><<<grid, NTHREADS, smem, s>>>(p.tmAh, p.tmAl, p.tmBh, p.tmBl, p.Kp / BK, ep, p.err);
    return cudaGetLastError();
}

}  // namespace

// Host preparation: B' hi/lo (once per model) and tensor maps.
int tc_plan_init(TcPlan& p, const DevModel& m, const cplx<double>* S_host) {
    p.N = m.N;
    p.nb = m.nb;
    p.nR = m.nR;
    p.PT = (m.nb == 10) ? 8 : 16;
    p.TN = 2 * m.nb * p.PT;  // 160 or 128 columns
    const int NN = m.N * m.N;
    p.n_tiles = (NN + p.PT - 1) / p.PT;
    p.Kp = ((2 * m.nR + BK - 1) / BK) * BK;
    p.ncolp = (size_t)p.n_tiles * p.TN;
    for (int i = 0; i < 9; ++i) p.C[i] = m.C[i];
    // per-block power-of-two scales: max |B| * sB <= 2^14
    double bmax[10] = {0};
    for (int r = 0; r < m.nR; ++r)
        for (int pr = 0; pr < NN; ++pr)
            for (int b = 0; b < m.nb; ++b) {
                const cplx<double> v = S_host[((size_t)r * NN + pr) * m.nb + b];
                bmax[b] = fmax(bmax[b], fmax(fabs(v.re), fabs(v.im)));
            }
    float sB[10];
    for (int b = 0; b < m.nb; ++b) {
        int e = 0;
        if (bmax[b] > 0) frexp(bmax[b], &e);  // bmax = f * 2^e, f in [0.5, 1)
        sB[b] = ldexpf(1.0f, 14 - e);
        p.inv_scale[b] = 1.0f / (sB[b] * kTcAScale);
    }
    std::vector<__half> bh((size_t)p.ncolp * p.Kp, __float2half(0.f)), bl((size_t)p.ncolp * p.Kp, __float2half(0.f));
    for (int t = 0; t < p.n_tiles; ++t)
        for (int b = 0; b < m.nb; ++b)
            for (int pl = 0; pl < p.PT; ++pl) {
                const int pair = t * p.PT + pl;
                if (pair >= NN) continue;
                const size_t col0 = (size_t)t * p.TN + (size_t)b * 2 * p.PT + 2 * pl;  // Re column; Im = col0 + 1
                for (int r = 0; r < m.nR; ++r) {
                    const cplx<double> v = S_host[((size_t)r * NN + pair) * m.nb + b];
                    const float sr = (float)(v.re * sB[b]), si = (float)(v.im * sB[b]);
                    const float vals[2][2] = {{sr, -si}, {si, sr}};  // [t][kappa parity]
                    for (int tt = 0; tt < 2; ++tt)
                        for (int kp = 0; kp < 2; ++kp) {
                            const float x = vals[tt][kp];
                            const __half h = __float2half_rn(x);
                            const __half l = __float2half_rn(x - __half2float(h));
                            const size_t idx = (col0 + tt) * p.Kp + 2 * r + kp;
                            bh[idx] = h;
                            bl[idx] = l;
                        }
                }
            }
    const size_t bytes = bh.size() * sizeof(__half);
    if (cudaMalloc(&p.Bh, bytes) != cudaSuccess) return MEPI_TC_NOMEM;
    if (cudaMalloc(&p.Bl, bytes) != cudaSuccess) return MEPI_TC_NOMEM;
    if (cudaMemcpy(p.Bh, bh.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) return MEPI_TC_CUDA;
    if (cudaMemcpy(p.Bl, bl.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) return MEPI_TC_CUDA;
    if (!encode_2d(&p.tmBh, p.Bh, p.Kp, p.ncolp, BK, p.TN)) return MEPI_TC_CUDA;
    if (!encode_2d(&p.tmBl, p.Bl, p.Kp, p.ncolp, BK, p.TN)) return MEPI_TC_CUDA;
    if (cudaMalloc(&p.err, sizeof(int)) != cudaSuccess) return MEPI_TC_NOMEM;
    if (cudaMemset(p.err, 0, sizeof(int)) != cudaSuccess) return MEPI_TC_CUDA;
    p.tau = m.tau;
    p.R = m.R;
    return 0;
}

int tc_plan_rows(TcPlan& p, int64_t rows_needed) {
    int64_t rows = ((rows_needed + BM - 1) / BM) * BM;
    if (rows <= p.rows_cap) {
        p.rows = rows;
        return 0;
    }
    if (p.Ah) cudaFree(p.Ah);
    if (p.Al) cudaFree(p.Al);
    p.Ah = p.Al = nullptr;
    p.rows_cap = 0;
    const size_t bytes = (size_t)rows * p.Kp * sizeof(__half);
    if (cudaMalloc(&p.Ah, bytes) != cudaSuccess) return MEPI_TC_NOMEM;
    if (cudaMalloc(&p.Al, bytes) != cudaSuccess) return MEPI_TC_NOMEM;
    if (!encode_2d(&p.tmAh, p.Ah, p.Kp, rows, BK, BM)) return MEPI_TC_CUDA;
    if (!encode_2d(&p.tmAl, p.Al, p.Kp, rows, BK, BM)) return MEPI_TC_CUDA;
    p.rows_cap = rows;
    p.rows = rows;
    return 0;
}

void tc_plan_free(TcPlan& p) {
    for (void* q : {(void*)p.Bh, (void*)p.Bl, (void*)p.Ah, (void*)p.Al, (void*)p.err})
        if (q) cudaFree(q);
    p = TcPlan();
}

cudaError_t launch_phase_split(const TcPlan& p, const KRange& kr, cudaStream_t s) {
    const int64_t total = (int64_t)p.rows * (p.Kp / 2);
    int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
    phase_split_kernel<<<blocks, 256, 0, s>>>(kr, p.R, p.nR, p.Kp, (int)p.rows, reinterpret_cast<__half2*>(p.Ah),
                                              reinterpret_cast<__half2*>(p.Al));
    return cudaGetLastError();
}

cudaError_t launch_ft_tc(const TcPlan& p, const KRange& kr, cplx<float>* W, cudaStream_t s) {
    if (kr.count <= 0) return cudaSuccess;
    if (p.nb == 10) return launch_tc_t<10, 160>(p, kr, W, s);
    return launch_tc_t<4, 128>(p, kr, W, s);
}

}  // namespace mepi
