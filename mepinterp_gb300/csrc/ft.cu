// Fourier sums H(k), H_a(k), A_a(k), Omega_ab(k) of FT_R_to_k
// (src/wann_interp.f90:151-384) as one batched complex GEMM
//     X[k][pair][blk] = sum_R exp(2 pi i k.R) S[R][pair][blk]
// followed by the tight-binding phase epilogue (per pair (n,m), with
// psi = exp(2 pi i k.(tau_m - tau_n)) and dt = C (tau_m - tau_n)):
//     H      = psi X_0
//     H_a    = i (psi X_a + dt_a H)                      a = x,y,z
//     A_b    = psi X_{3+b}
//     Om_ab  = i (psi X_Q + dt_a A_b - dt_b A_a)         Q = (x,y),(x,z),(y,z)
// which is the reference's per-element angle 2 pi k.(R + tau_m - tau_n)
// factorised; the Wannier convention is tau = 0.
//
// This is the all-FP64 SIMT form: FP64 FMA throughput bounds it.  Each thread
// owns one (n,m) pair for two k-points and keeps all stack blocks of that pair
// in registers, so the epilogue runs in registers and the W-gauge blocks are
// written once, coalesced along m.
#include "mepi_internal.cuh"

namespace mepi {

namespace {
constexpr int TK = 64;   // k-points per CTA
constexpr int TP = 8;    // (n,m) pairs per CTA
constexpr int RT = 8;    // R vectors per shared-memory stage
constexpr int NT = 256;  // threads

template <typename T, int NB>
__global__ void __launch_bounds__(NT) ft_simt_kernel(DevModel m, KRange kr, cplx<T>* __restrict__ W) {
    __shared__ cplx<double> Ps[RT][TK];
    __shared__ cplx<double> Ss[RT][TP * NB];
    __shared__ double ks[TK][3];
    const int tid = threadIdx.x;
    const int NN = m.N * m.N;
    const int64_t k0 = (int64_t)blockIdx.x * TK;
    const int p0 = blockIdx.y * TP;
    const int pl = tid % TP, kg = tid / TP;
    if (tid < TK) {
        double k[3] = {0.0, 0.0, 0.0};
        int64_t i = k0 + tid;
        if (i < kr.count) {
            if (kr.kpts) {
                k[0] = kr.kpts[3 * i]; k[1] = kr.kpts[3 * i + 1]; k[2] = kr.kpts[3 * i + 2];
            } else {
                mp_kpt(kr.mp, k_of(kr, i), k);
            }
        }
        ks[tid][0] = k[0]; ks[tid][1] = k[1]; ks[tid][2] = k[2];
    }
    cplx<double> acc0[NB], acc1[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) { acc0[b] = mk(0.0, 0.0); acc1[b] = mk(0.0, 0.0); }

    for (int r0 = 0; r0 < m.nR; r0 += RT) {
        __syncthreads();
        for (int e = tid; e < TK * RT; e += NT) {
            int rr = e / TK, kk = e % TK, R = r0 + rr;
            cplx<double> v = mk(0.0, 0.0);
            if (R < m.nR) {
                double x = ks[kk][0] * m.R[3 * R] + ks[kk][1] * m.R[3 * R + 1] + ks[kk][2] * m.R[3 * R + 2];
                double s, c;
                sincospi(2.0 * x, &s, &c);
                v = mk(c, s);
            }
            Ps[rr][kk] = v;
        }
        for (int e = tid; e < RT * TP * NB; e += NT) {
            int rr = e / (TP * NB), q = e % (TP * NB), R = r0 + rr, pair = p0 + q / NB;
            cplx<double> v = mk(0.0, 0.0);
            if (R < m.nR && pair < NN) v = m.S[((size_t)R * NN + p0) * NB + q];
            Ss[rr][q] = v;
        }
        __syncthreads();
#pragma unroll
        for (int rr = 0; rr < RT; ++rr) {
            cplx<double> pa = Ps[rr][kg], pb = Ps[rr][kg + TK / 2];
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                cplx<double> s = Ss[rr][pl * NB + b];
                fma_c(acc0[b], pa, s);
                fma_c(acc1[b], pb, s);
            }
        }
    }
    const int pair = p0 + pl;
    const int nbo = NB;
    if (pair < NN) {
        int64_t i0 = k0 + kg, i1 = k0 + kg + TK / 2;
        if (i0 < kr.count) {
            double k[3] = {ks[kg][0], ks[kg][1], ks[kg][2]};
            ft_epilogue<T, NB>(m, k, pair, acc0, W + (size_t)i0 * nbo * NN, NN);
        }
        if (i1 < kr.count) {
            double k[3] = {ks[kg + TK / 2][0], ks[kg + TK / 2][1], ks[kg + TK / 2][2]};
            ft_epilogue<T, NB>(m, k, pair, acc1, W + (size_t)i1 * nbo * NN, NN);
        }
    }
}
// H(k) alone in FP64 for the mixed form's energy refinement: the same
// contraction restricted to stack block 0 (read with the stack's block stride),
// 8 k-points x 1 pair per thread, tau phase applied, Hdf[k][n][m] written as
// double-FP32 pairs (the FP64 value split once).
constexpr int HK = 64, HP = 32;
__global__ void __launch_bounds__(NT) ft_h64_kernel(DevModel m, KRange kr, float4* __restrict__ Hdf) {
    __shared__ cplx<double> Ps[RT][HK];
    __shared__ cplx<double> Ss[RT][HP];
    __shared__ double ks[HK][3];
    const int tid = threadIdx.x;
    const int NN = m.N * m.N;
    const int64_t k0 = (int64_t)blockIdx.x * HK;
    const int p0 = blockIdx.y * HP;
    const int pl = tid % HP, kg = tid / HP;  // kg 0..7 -> k = kg + 8 j
    if (tid < HK) {
        double k[3] = {0.0, 0.0, 0.0};
        int64_t i = k0 + tid;
        if (i < kr.count) {
            if (kr.kpts) {
                k[0] = kr.kpts[3 * i]; k[1] = kr.kpts[3 * i + 1]; k[2] = kr.kpts[3 * i + 2];
            } else {
                mp_kpt(kr.mp, k_of(kr, i), k);
            }
        }
        ks[tid][0] = k[0]; ks[tid][1] = k[1]; ks[tid][2] = k[2];
    }
    cplx<double> acc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = mk(0.0, 0.0);
    for (int r0 = 0; r0 < m.nR; r0 += RT) {
        __syncthreads();
        for (int e = tid; e < HK * RT; e += NT) {
            int rr = e / HK, kk = e % HK, R = r0 + rr;
            cplx<double> v = mk(0.0, 0.0);
            if (R < m.nR) {
                double x = ks[kk][0] * m.R[3 * R] + ks[kk][1] * m.R[3 * R + 1] + ks[kk][2] * m.R[3 * R + 2];
                double sn, cs;
                sincospi(2.0 * x, &sn, &cs);
                v = mk(cs, sn);
            }
            Ps[rr][kk] = v;
        }
        for (int e = tid; e < RT * HP; e += NT) {
            int rr = e / HP, q = e % HP, R = r0 + rr, pair = p0 + q;
            cplx<double> v = mk(0.0, 0.0);
            if (R < m.nR && pair < NN) v = m.S[((size_t)R * NN + pair) * m.nb];
            Ss[rr][q] = v;
        }
        __syncthreads();
#pragma unroll
        for (int rr = 0; rr < RT; ++rr) {
            const cplx<double> s = Ss[rr][pl];
#pragma unroll
            for (int j = 0; j < 8; ++j) fma_c(acc[j], Ps[rr][kg + 8 * j], s);
        }
    }
    const int pair = p0 + pl;
    if (pair >= NN) return;
    const int n = pair / m.N, mm = pair % m.N;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int kk = kg + 8 * j;
        const int64_t i = k0 + kk;
        if (i >= kr.count) continue;
        cplx<double> psi = mk(1.0, 0.0);
        if (m.has_tau) {
            double x = 0.0;
            for (int c = 0; c < 3; ++c) x += ks[kk][c] * (m.tau[mm * 3 + c] - m.tau[n * 3 + c]);
            double sn, cs;
            sincospi(2.0 * x, &sn, &cs);
            psi = mk(cs, sn);
        }
        const cplx<double> x = psi * acc[j];
        const float hr = (float)x.re, hi = (float)x.im;
        Hdf[(size_t)i * NN + pair] = make_float4(hr, hi, (float)(x.re - (double)hr), (float)(x.im - (double)hi));
    }
}

}  // namespace

cudaError_t launch_ft_h64(const DevModel& m, const KRange& kr, float4* Hdf, cudaStream_t s) {
    if (kr.count <= 0) return cudaSuccess;
    const int NN = m.N * m.N;
    dim3 grid((unsigned)((kr.count + HK - 1) / HK), (unsigned)((NN + HP - 1) / HP));
    ft_h64_kernel<<<grid, NT, 0, s>>>(m, kr, Hdf);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_ft_simt(const DevModel& m, const KRange& kr, cplx<T>* W, cudaStream_t s) {
    if (kr.count <= 0) return cudaSuccess;
    const int NN = m.N * m.N;
    dim3 grid((unsigned)((kr.count + TK - 1) / TK), (unsigned)((NN + TP - 1) / TP));
    if (m.nb == 10)
        ft_simt_kernel<T, 10><<<grid, NT, 0, s>>>(m, kr, W);
    else
        ft_simt_kernel<T, 4><<<grid, NT, 0, s>>>(m, kr, W);
    return cudaGetLastError();
}

template cudaError_t launch_ft_simt<double>(const DevModel&, const KRange&, cplx<double>*, cudaStream_t);
template cudaError_t launch_ft_simt<float>(const DevModel&, const KRange&, cplx<float>*, cudaStream_t);

}  // namespace mepi
