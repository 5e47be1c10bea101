// Band sums of one rank's k-points; each k-point's tensors are formed in the
// working precision T and accumulated over k in FP64:
//   kubo_ahc_tens (src/kubo.f90:37-78)
//       curv(i,j,n) = -2 sum_{m!=n} Im(V_i(n,m) V_j(m,n)) / (E_m - E_n)^2
//       ahc(i,j,e) -= sum_n curv(i,j,n) f(e,n)
//   mep_niu_IC / kubo_mep_IC (src/mep_niu.f90:102-159, src/kubo_mep.f90:100-149)
//       F2(i,j,n0) = -sum_{n,m != n0} Re(V_i(n0,n) (V(n,m) x V(m,n0))_j)
//                                     / ((E0-En)^2 (E0-Em))
//   mep_niu_LC / kubo_mep_LC (src/mep_niu.f90:47-99, src/kubo_mep.f90:51-97)
//       F3(i,j,n0) = sum_{n != n0} Re(V_i(n0,n) (V(n,n0) x V(n0,n0))_j) / (E0-En)^3
//   mep_niu_CS / kubo_mep_CS: per-band value csv(n0) from the gauge kernel.
// (x is the Levi-Civita contraction sum_kl eps_jkl a_k b_l.)  The Niu sums run
// over n0 < valence_bands and skip terms whose product denominator satisfies
// |den| <= kuboTol, exactly as the reference; the Kubo sums run over all n0,
// weight by f(e,n0) and have no guard (D9).
//
// Work split: the CTA stages V (row stride N+1) in shared memory; warp w
// handles bands n0 = w, w + nwarps, ...; lane l handles n = l, l+32 and loops
// over m for the IC contraction, then the warp reduces the per-band tensors.
// The Fermi contraction runs one thread (nE >= 64) or one warp (nE < 64) per
// Fermi energy.  A CTA owns one FP64 accumulator slice for its whole k stripe
// (k = blockIdx.x, blockIdx.x + gridDim.x, ...), so the final reduction over
// slices runs in a fixed order and the result is deterministic.
#include <cmath>
#include <mutex>

#include "../../include/mepi.h"
#include "mepi_internal.cuh"

namespace mepi {

namespace {

template <typename T>
__device__ __forceinline__ T fd_stat(double e_band, double e_fermi, double T_kelvin) {  // src/statistics.f90:65-90
    if (T_kelvin > kMinTemp) {
        const T x = (T)((e_band - e_fermi) / (kKbEhK * T_kelvin));
        return (T)1 / ((T)1 + exp(x));
    }
    return (e_band < e_fermi) ? (T)1 : (T)0;
}

// cross(a, b)_j = sum_kl eps_jkl a_k b_l
template <typename T>
__device__ __forceinline__ void cross3(const cplx<T> a[3], const cplx<T> b[3], cplx<T> out[3]) {
    out[0] = a[1] * b[2] - a[2] * b[1];
    out[1] = a[2] * b[0] - a[0] * b[2];
    out[2] = a[0] * b[1] - a[1] * b[0];
}

// acc -= a * b
template <typename T>
__device__ __forceinline__ void fms_c(cplx<T>& acc, cplx<T> a, cplx<T> b) {
    acc.re = fma(-a.re, b.re, acc.re); acc.re = fma(a.im, b.im, acc.re);
    acc.im = fma(-a.re, b.im, acc.im); acc.im = fma(-a.im, b.re, acc.im);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Fermi contraction of the per-band curvature, -sum_n curv(n) f(n): FP64 in
// the FP64 form; double-FP32 in the FP32 form (curvature stored as leading
// part + remainder), so that no FP64 instruction runs per k-point there.
template <typename T> struct CurvSum;
template <> struct CurvSum<double> {
    double v;
    __device__ __forceinline__ void zero() { v = 0.0; }
    __device__ __forceinline__ void sub(const double* curv, const float*, const float*, int i, double f) {
        v -= curv[i] * f;
    }
    __device__ __forceinline__ void warp_reduce() { v = warp_sum(v); }
    __device__ __forceinline__ double value() const { return v; }
};
template <> struct CurvSum<float> {
    DF v;
    __device__ __forceinline__ void zero() { v = DF{0.f, 0.f}; }
    __device__ __forceinline__ void sub(const double*, const float* cs, const float* cc, int i, float f) {
        df_add_prod(v, -cs[i], f);
        v.c = __fmaf_rn(-cc[i], f, v.c);
    }
    __device__ __forceinline__ void warp_reduce() { v = df_warp_sum(v); }
    __device__ __forceinline__ double value() const { return (double)v.s + (double)v.c; }
};

// kGemm (FP32 form, N <= 32): the IC contraction of every (n, n0) pair,
//     G_j(n, n0) = sum_{m != n0} (V(n,m) x W(m,n0))_j,  W(m,n0) = V(m,n0) / (E0 - Em),
// is formed once per k-point as a register-tiled CUDA-core GEMM over m (2 x 2
// (n, n0) tiles per thread, 24 FMA per (n, n0, m)) instead of inside the band
// loop.  The Niu sum needs the same contraction without the terms whose product
// denominator |(E0-En)^2 (E0-Em)| is within kuboTol: it equals G unless the
// band nearest to n0 already fails that test (the rounded product is monotone
// in |E0-Em|), and only for those (n0, n) pairs is it summed directly.
constexpr int kMaskCap = 256;   // masked Niu pairs summed by whole warps per k-point

// sum over the aligned group of 8 lanes
__device__ __forceinline__ float sum8(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    return v;
}
__device__ __forceinline__ DF df_sum8(DF v) {
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        const DF w{__shfl_xor_sync(0xffffffffu, v.s, o), __shfl_xor_sync(0xffffffffu, v.c, o)};
        v = df_sum(v, w);
    }
    return v;
}

// Band-pair phase of the FP32 form for N <= 32, after the IC contraction G
// (see bandsum_kernel): per band n0 the AHC curvature, the LC and IC terms,
// Kubo (every n0) and Niu (n0 < valence_bands, kuboTol guard).
//  1. the (n0, n) Niu pairs whose kuboTol window is not empty go to a compact
//     list; a warp sums each one over m (lane = m) with the guard applied;
//  2. eight threads per band n0 walk n = part, part + 8, ... and reduce their
//     per-band tensors over the group of eight (three shuffle levels).
__device__ __noinline__ void bandsum_pairs_gemm(const DevModel& md, const JobDev& jb, int N, int ld,
                                                const cplx<float>* Vs, const cplx<float>* Ws, const cplx<float>* Gs,
                                                cplx<float>* GVl, const float* dmin, int* s_list, short* s_map,
                                                int& s_cnt, const float* Dt, const float* Iv, float* curvS,
                                                float* curvC, float* icn, float* lcn, float* icv, float* lcv) {
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    const int nval = jb.nval;
    const float ttol = (float)md.kubo_tol;
    auto V = [&](int a, int n, int m) -> cplx<float> { return Vs[(a * N + n) * ld + m]; };
    auto W = [&](int a, int m, int n0) -> cplx<float> { return Ws[(a * 32 + m) * 33 + n0]; };
    const bool mep = jb.do_mep && nval > 0;
    if (tid == 0) s_cnt = 0;
    __syncthreads();
    if (mep) {
        for (int t = tid; t < nval * N; t += nt) {
            const int n0 = t / N, n = t - n0 * N;
            short id = -1;
            if (n != n0) {
                const float d0n = Dt[n0 * ld + n], a2 = d0n * d0n;
                if (!(fabsf(a2 * dmin[n0]) > ttol)) {
                    const int e = atomicAdd(&s_cnt, 1);
                    if (e < kMaskCap) {
                        s_list[e] = (n0 << 8) | n;
                        id = (short)e;
                    } else {
                        id = -2;
                    }
                }
            }
            s_map[n0 * 32 + n] = id;
        }
    }
    __syncthreads();
    const int cnt = mep ? min(s_cnt, kMaskCap) : 0;
    for (int e = warp; e < cnt; e += nwarps) {
        const int n0 = s_list[e] >> 8, n = s_list[e] & 255;
        const float d0n = Dt[n0 * ld + n], a2 = d0n * d0n;
        cplx<float> x[3] = {mk(0.f, 0.f), mk(0.f, 0.f), mk(0.f, 0.f)};
        const int m = lane;
        if (m < N && m != n0 && fabsf(a2 * Dt[n0 * ld + m]) > ttol) {
            cplx<float> vnm[3], wmo[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                vnm[c] = V(c, n, m);
                wmo[c] = W(c, m, n0);
            }
            cross3(vnm, wmo, x);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) x[c] = mk(warp_sum(x[c].re), warp_sum(x[c].im));
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) GVl[e * 3 + c] = x[c];
        }
    }
    __syncthreads();
    // eight threads per band n0
    const int n0 = tid >> 3, part = tid & 7;
    const bool live = n0 < N;
    const bool niu = live && (n0 < nval) && jb.do_mep;
    DF s_curv[9];
    float s_ic[9], s_lc[9], s_icv[9], s_lcv[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        s_curv[q] = DF{0.f, 0.f};
        s_ic[q] = s_lc[q] = s_icv[q] = s_lcv[q] = 0.f;
    }
    if (live) {
        cplx<float> vnn[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) vnn[c] = V(c, n0, n0);
        for (int n = part; n < N; n += 8) {
            if (n == n0) continue;
            const float d0n = Dt[n0 * ld + n];   // E0 - En
            const float i0n = Iv[n0 * ld + n];   // 1 / (E0 - En)
            cplx<float> vi[3], vk[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) { vi[c] = V(c, n0, n); vk[c] = V(c, n, n0); }
            if (jb.do_ahc) {
                // the pair term formed once from (a, b) = (min, max): + to band a, - to band b
                const int a = n0 < n ? n0 : n, b = n0 < n ? n : n0;
                const float iab = Iv[a * ld + b];
                const float w = (n0 < n ? -2.f : 2.f) * iab * iab;
                cplx<float> va[3], vb[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) { va[c] = V(c, a, b); vb[c] = V(c, b, a); }
#pragma unroll
                for (int j = 0; j < 3; ++j)
#pragma unroll
                    for (int i = 0; i < 3; ++i) df_add(s_curv[i + 3 * j], w * (va[i] * vb[j]).im);
            }
            {   // LC
                cplx<float> x[3];
                cross3(vk, vnn, x);
                const float den3 = d0n * d0n * d0n, i3 = i0n * i0n * i0n;
                const bool kubo_ok = jb.do_kubo, niu_ok = niu && (fabsf(den3) > ttol);
                if (kubo_ok || niu_ok) {
#pragma unroll
                    for (int j = 0; j < 3; ++j)
#pragma unroll
                        for (int i = 0; i < 3; ++i) {
                            const float v = (vi[i] * x[j]).re * i3;
                            if (kubo_ok) s_lc[i + 3 * j] += v;
                            if (niu_ok) s_lcv[i + 3 * j] += v;
                        }
                }
            }
            if (jb.do_kubo || niu) {   // IC from the contraction G
                cplx<float> g[3], gv[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    g[c] = Gs[(c * 32 + n) * 33 + n0];
                    gv[c] = mk(0.f, 0.f);
                }
                if (niu) {
                    const int id = s_map[n0 * 32 + n];
                    if (id == -1) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) gv[c] = g[c];
                    } else if (id >= 0) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) gv[c] = GVl[id * 3 + c];
                    } else {   // beyond the list's capacity: the guarded sum here
                        const float a2 = d0n * d0n;
                        for (int m = 0; m < N; ++m) {
                            if (m == n0 || !(fabsf(a2 * Dt[n0 * ld + m]) > ttol)) continue;
                            cplx<float> vnm[3], wmo[3], x[3];
#pragma unroll
                            for (int c = 0; c < 3; ++c) {
                                vnm[c] = V(c, n, m);
                                wmo[c] = W(c, m, n0);
                            }
                            cross3(vnm, wmo, x);
#pragma unroll
                            for (int c = 0; c < 3; ++c) gv[c] = gv[c] + x[c];
                        }
                    }
                }
                const float ainv = i0n * i0n;
#pragma unroll
                for (int j = 0; j < 3; ++j)
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        s_ic[i + 3 * j] -= (vi[i] * g[j]).re * ainv;
                        s_icv[i + 3 * j] -= (vi[i] * gv[j]).re * ainv;
                    }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const DF rf = df_sum8(s_curv[q]);
        const float b = sum8(s_ic[q]), c = sum8(s_lc[q]), d = sum8(s_icv[q]), e = sum8(s_lcv[q]);
        if (live && part == 0) {
            curvS[q * N + n0] = rf.s;
            curvC[q * N + n0] = rf.c;
            icn[q * N + n0] = b;
            lcn[q * N + n0] = c;
            icv[q * kMaxN + n0] = d;
            lcv[q * kMaxN + n0] = e;
        }
    }
}

template <typename T, bool kGemm>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 2 : 1) bandsum_kernel(DevModel md, JobDev jb, int64_t nk, const double* __restrict__ Eg,
                                                      const cplx<T>* __restrict__ Vg, const T* __restrict__ CSVg,
                                                      const int* __restrict__ skip, double* __restrict__ partials,
                                                      int use_tab) {
    extern __shared__ unsigned char smem_raw[];
    const int N = md.N, NN = N * N, ld = N + 1;
    const int nval = jb.nval, nE = jb.nE;
    cplx<T>* Vs = reinterpret_cast<cplx<T>*>(smem_raw);          // [3][N][ld]
    double* curv = reinterpret_cast<double*>(Vs + 3 * N * ld);    // [9][N] AHC curvature per band: FP64, or
    float* curvS = reinterpret_cast<float*>(curv);                 // in the FP32 form the leading parts [9][N]
    float* curvC = curvS + 9 * N;                                  // and remainders [9][N] (same bytes)
    double* Es = curv + 9 * N;                                    // [kMaxN] energies (FP64)
    T* icn = reinterpret_cast<T*>(Es + kMaxN);                    // [9][N] Kubo IC per band
    T* lcn = icn + 9 * N;                                         // [9][N] Kubo LC per band
    T* icv = lcn + 9 * N;                                         // [9][kMaxN] Niu IC
    T* lcv = icv + 9 * kMaxN;                                     // [9][kMaxN] Niu LC
    T* Cs = lcv + 9 * kMaxN;                                      // [kMaxN]
    T* Dt = Cs + kMaxN;                                           // [N][ld] E_a - E_b (difference formed in FP64;
                                                                  // rows padded: band-parallel walks conflict-free)
    T* Iv = Dt + N * ld;                                          // [N][ld] 1 / (E_a - E_b), 0 on the diagonal
    // kGemm: W and G as [3][32][33] complex, and the nearest-band distance per band
    cplx<T>* Ws = reinterpret_cast<cplx<T>*>((reinterpret_cast<uintptr_t>(Iv + N * ld) + 15) & ~uintptr_t(15));
    cplx<T>* Gs = Ws + 3 * 32 * 33;
    cplx<T>* GVl = Gs + 3 * 32 * 33;                              // [kMaskCap][3] masked Niu IC sums
    T* dmin = reinterpret_cast<T*>(GVl + 3 * kMaskCap);
    int* s_list = reinterpret_cast<int*>(dmin + 32);              // [kMaskCap] (n0 << 8) | n
    short* s_map = reinterpret_cast<short*>(s_list + kMaskCap);   // [32][32] list index, -1 none, -2 over cap
    __shared__ int s_cnt;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    const AccLayout L{nE, nval, jb.nW};
    double* P = partials + (size_t)blockIdx.x * L.size();
    const T ttol = (T)md.kubo_tol;

    for (int64_t k = blockIdx.x; k < nk; k += gridDim.x) {
        // the next k-point's velocities into L2 while this one is summed
        if (tid < 3 && k + gridDim.x < nk)
            l2_prefetch(Vg + ((size_t)(k + gridDim.x) * 3 + tid) * NN, (uint32_t)(NN * sizeof(cplx<T>)));
        if (skip && skip[k]) continue;
        __syncthreads();
        for (int e = tid; e < 3 * NN; e += nt) {
            int a = e / NN, r = e % NN, n = r / N, m = r % N;
            Vs[(a * N + n) * ld + m] = Vg[(size_t)k * 3 * NN + e];
        }
        for (int n = tid; n < N; n += nt) {
            Es[n] = Eg[(size_t)k * N + n];
            Cs[n] = CSVg ? CSVg[(size_t)k * N + n] : (T)0;
        }
        __syncthreads();
        if (use_tab) {
            if constexpr (sizeof(T) == 4) {
                // the FP64 differences rounded to FP32, formed from FP32 hi/lo energies
                __shared__ float s_Eh[kMaxN], s_El[kMaxN];
                for (int n = tid; n < N; n += nt) {
                    s_Eh[n] = (float)Es[n];
                    s_El[n] = (float)(Es[n] - (double)s_Eh[n]);
                }
                __syncthreads();
                for (int e = tid; e < NN; e += nt) {
                    const int a = e / N, b = e % N;
                    float d, dl;
                    df_diff(s_Eh[a], s_El[a], s_Eh[b], s_El[b], d, dl);
                    Dt[a * ld + b] = d;
                    Iv[a * ld + b] = (a == b) ? 0.f : 1.f / d;
                }
            } else {
                for (int e = tid; e < NN; e += nt) {
                    const int a = e / N, b = e % N;
                    const T d = (T)(Es[a] - Es[b]);
                    Dt[a * ld + b] = d;
                    Iv[a * ld + b] = (a == b) ? (T)0 : (T)1 / d;
                }
            }
        }
        __syncthreads();
        auto V = [&](int a, int n, int m) -> cplx<T> { return Vs[(a * N + n) * ld + m]; };
        if constexpr (kGemm) {
            if (jb.do_kubo || (jb.do_mep && nval > 0)) {
                for (int e = tid; e < 3 * 32 * 32; e += nt) {
                    const int l = e >> 10, m = (e >> 5) & 31, n0 = e & 31;
                    cplx<T> w = mk((T)0, (T)0);
                    // 1 / (E_n0 - E_m) = -(1 / (E_m - E_n0)) to the bit (the differences are
                    // antisymmetric and the reciprocal sign-symmetric): read along the row
                    // m, so that the lanes (n0) meet no bank conflict
                    if (m < N && n0 < N && m != n0) w = -Iv[m * ld + n0] * V(l, m, n0);
                    Ws[(l * 32 + m) * 33 + n0] = w;
                }
                for (int n0 = tid; n0 < N; n0 += nt) {
                    T dm = (T)1e30;
                    for (int m = 0; m < N; ++m)
                        if (m != n0) dm = fmin(dm, (T)fabs(Dt[n0 * ld + m]));
                    dmin[n0] = dm;
                }
                __syncthreads();
                for (int t = tid; t < 256; t += nt) {
                    // 2 x 2 tiles: rows nb, nb + 1 and columns ob, ob + 16 (consecutive
                    // lanes on consecutive columns: conflict-free Ws loads, Gs stores)
                    const int nb = 2 * (t >> 4), ob = t & 15;
                    cplx<T> acc[2][2][3];
#pragma unroll
                    for (int i = 0; i < 2; ++i)
#pragma unroll
                        for (int jj = 0; jj < 2; ++jj)
#pragma unroll
                            for (int c = 0; c < 3; ++c) acc[i][jj][c] = mk((T)0, (T)0);
                    for (int m = 0; m < N; ++m) {
                        cplx<T> a[2][3], b[2][3];
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
#pragma unroll
                            for (int i = 0; i < 2; ++i) a[i][c] = (nb + i < N) ? V(c, nb + i, m) : mk((T)0, (T)0);
#pragma unroll
                            for (int jj = 0; jj < 2; ++jj) b[jj][c] = Ws[(c * 32 + m) * 33 + ob + 16 * jj];
                        }
#pragma unroll
                        for (int i = 0; i < 2; ++i)
#pragma unroll
                            for (int jj = 0; jj < 2; ++jj) {
                                // (a x b)_j = a_k b_l - a_l b_k, (j,k,l) cyclic
                                fma_c(acc[i][jj][0], a[i][1], b[jj][2]);
                                fms_c(acc[i][jj][0], a[i][2], b[jj][1]);
                                fma_c(acc[i][jj][1], a[i][2], b[jj][0]);
                                fms_c(acc[i][jj][1], a[i][0], b[jj][2]);
                                fma_c(acc[i][jj][2], a[i][0], b[jj][1]);
                                fms_c(acc[i][jj][2], a[i][1], b[jj][0]);
                            }
                    }
#pragma unroll
                    for (int i = 0; i < 2; ++i)
#pragma unroll
                        for (int jj = 0; jj < 2; ++jj)
#pragma unroll
                            for (int c = 0; c < 3; ++c) Gs[(c * 32 + nb + i) * 33 + ob + 16 * jj] = acc[i][jj][c];
                }
                __syncthreads();
            }
        }
        // energy differences (formed in FP64) and their inverses: tabulated when
        // they fit in shared memory, else formed on the fly
        auto dE = [&](int a, int b) -> T { return use_tab ? Dt[a * ld + b] : (T)(Es[a] - Es[b]); };
        auto iE = [&](int a, int b) -> T {
            return use_tab ? Iv[a * ld + b] : (a == b ? (T)0 : (T)1 / (T)(Es[a] - Es[b]));
        };

        if constexpr (kGemm && sizeof(T) == 4) {
            bandsum_pairs_gemm(md, jb, N, ld, Vs, Ws, Gs, GVl, dmin, s_list, s_map, s_cnt, Dt, Iv, curvS, curvC, icn,
                               lcn, icv, lcv);
        }
        for (int n0 = warp; n0 < (kGemm ? 0 : N); n0 += nwarps) {
            const bool niu = (n0 < nval) && jb.do_mep;
            // per-band curvature: FP64 in the FP64 form, double-FP32 (TwoSum) in
            // the FP32 form, so that the pair terms of two occupied bands still
            // cancel to well below the FP32 rounding of one term
            double s_curv[9];
            DF s_curvf[9];
            T s_ic[9], s_lc[9], s_icv[9], s_lcv[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                s_curv[q] = 0.0;
                s_curvf[q] = DF{0.f, 0.f};
                s_ic[q] = s_lc[q] = s_icv[q] = s_lcv[q] = (T)0;
            }
            cplx<T> vnn[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) vnn[c] = V(c, n0, n0);
            for (int n = lane; n < N; n += 32) {
                if (n == n0) continue;
                const T d0n = dE(n0, n);   // E0 - En
                const T i0n = iE(n0, n);   // 1 / (E0 - En)
                cplx<T> vi[3], vk[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) { vi[c] = V(c, n0, n); vk[c] = V(c, n, n0); }
                // AHC: curv(i,j,n0) = -2 sum_n Im(V_i(n0,n) V_j(n,n0)) / (En - E0)^2.  The pair term is
                // formed once from the ordered pair (a,b) = (min, max) and enters band a with + and band
                // b with -, so two bands of equal occupation cancel exactly in the Fermi contraction.
                if (jb.do_ahc) {
                    const int a = n0 < n ? n0 : n, b = n0 < n ? n : n0;
                    const T iab = iE(a, b);
                    const T w = (n0 < n ? (T)-2 : (T)2) * iab * iab;
                    cplx<T> va[3], vb[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) { va[c] = V(c, a, b); vb[c] = V(c, b, a); }
#pragma unroll
                    for (int j = 0; j < 3; ++j)
#pragma unroll
                        for (int i = 0; i < 3; ++i) {
                            const T term = w * (va[i] * vb[j]).im;
                            if constexpr (sizeof(T) == 4) df_add(s_curvf[i + 3 * j], term);
                            else s_curv[i + 3 * j] += (double)term;
                        }
                }
                // LC
                {
                    cplx<T> x[3];
                    cross3(vk, vnn, x);
                    const T den3 = d0n * d0n * d0n;
                    const T i3 = i0n * i0n * i0n;
                    bool kubo_ok = jb.do_kubo;
                    bool niu_ok = niu && (fabs(den3) > ttol);
                    if (kubo_ok || niu_ok) {
#pragma unroll
                        for (int j = 0; j < 3; ++j)
#pragma unroll
                            for (int i = 0; i < 3; ++i) {
                                T v = (vi[i] * x[j]).re * i3;
                                if (kubo_ok) s_lc[i + 3 * j] += v;
                                if (niu_ok) s_lcv[i + 3 * j] += v;
                            }
                    }
                }
                // IC: g_j = sum_{m != n0} (V(n,m) x V(m,n0))_j / (E0 - Em)
                if (jb.do_kubo || niu) {
                    cplx<T> g[3], gv[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) g[c] = gv[c] = mk((T)0, (T)0);
                    const T a2 = d0n * d0n;
                    if constexpr (kGemm) {
#pragma unroll
                        for (int c = 0; c < 3; ++c) g[c] = Gs[(c * 32 + n) * 33 + n0];
                        if (niu) {
                            if (fabs(a2 * dmin[n0]) > ttol) {
#pragma unroll
                                for (int c = 0; c < 3; ++c) gv[c] = g[c];
                            } else {
                                for (int m = 0; m < N; ++m) {
                                    if (m == n0 || !(fabs(a2 * dE(n0, m)) > ttol)) continue;
                                    cplx<T> vnm[3], wmo[3], x[3];
#pragma unroll
                                    for (int c = 0; c < 3; ++c) {
                                        vnm[c] = V(c, n, m);
                                        wmo[c] = Ws[(c * 32 + m) * 33 + n0];
                                    }
                                    cross3(vnm, wmo, x);
#pragma unroll
                                    for (int c = 0; c < 3; ++c) gv[c] = gv[c] + x[c];
                                }
                            }
                        }
                    }
                    for (int m = 0; m < (kGemm ? 0 : N); ++m) {
                        if (m == n0) continue;
                        cplx<T> vnm[3], vmo[3], x[3];
#pragma unroll
                        for (int c = 0; c < 3; ++c) { vnm[c] = V(c, n, m); vmo[c] = V(c, m, n0); }
                        cross3(vnm, vmo, x);
                        const T b = iE(n0, m);
#pragma unroll
                        for (int c = 0; c < 3; ++c) g[c] = g[c] + b * x[c];
                        if (niu && fabs(a2 * dE(n0, m)) > ttol) {
#pragma unroll
                            for (int c = 0; c < 3; ++c) gv[c] = gv[c] + b * x[c];
                        }
                    }
                    const T ainv = i0n * i0n;
#pragma unroll
                    for (int j = 0; j < 3; ++j)
#pragma unroll
                        for (int i = 0; i < 3; ++i) {
                            s_ic[i + 3 * j] -= (vi[i] * g[j]).re * ainv;
                            s_icv[i + 3 * j] -= (vi[i] * gv[j]).re * ainv;
                        }
                }
            }
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                DF rf{0.f, 0.f};
                double a = 0.0;
                if constexpr (sizeof(T) == 4) rf = df_warp_sum(s_curvf[q]);
                else a = warp_sum(s_curv[q]);
                T b = warp_sum(s_ic[q]), c = warp_sum(s_lc[q]);
                T d = warp_sum(s_icv[q]), e = warp_sum(s_lcv[q]);
                if (lane == 0) {
                    if constexpr (sizeof(T) == 4) {
                        curvS[q * N + n0] = rf.s;
                        curvC[q * N + n0] = rf.c;
                    } else {
                        curv[q * N + n0] = a;
                    }
                    icn[q * N + n0] = b;
                    lcn[q * N + n0] = c;
                    if (n0 < kMaxN) { icv[q * kMaxN + n0] = d; lcv[q * kMaxN + n0] = e; }
                }
            }
        }
        __syncthreads();
        // Niu MEP: band resolved, no occupation weight
        if (jb.do_mep) {
            for (int t = tid; t < 9 * nval; t += nt) {
                int q = t % 9, n0 = t / 9;
                P[L.mic_off() + q + 9 * n0] += (double)icv[q * kMaxN + n0];
                P[L.mlc_off() + q + 9 * n0] += (double)lcv[q * kMaxN + n0];
                if (q == 0 || q == 4 || q == 8) P[L.mcs_off() + q + 9 * n0] += (double)Cs[n0];
            }
        }
        // Fermi contraction
        if (nE >= 64) {
            for (int e = tid; e < nE; e += nt) {
                const double ef = jb.ef[e];
                T ne = 0, ki[9], kl[9], kc = 0;
                CurvSum<T> a[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) { a[q].zero(); ki[q] = kl[q] = 0; }
                for (int n = 0; n < N; ++n) {
                    const T f = fd_stat<T>(Es[n], ef, jb.T_kelvin);
                    ne += f;
                    kc += f * Cs[n];
#pragma unroll
                    for (int q = 0; q < 9; ++q) {
                        a[q].sub(curv, curvS, curvC, q * N + n, f);
                        ki[q] += icn[q * N + n] * f;
                        kl[q] += lcn[q * N + n] * f;
                    }
                }
                P[L.ne_off() + e] += ne;
                if (jb.do_ahc)
                    for (int q = 0; q < 9; ++q) P[L.ahc_off() + q + 9 * e] += a[q].value();
                if (jb.do_kubo) {
                    for (int q = 0; q < 9; ++q) {
                        P[L.kic_off() + q + 9 * e] += ki[q];
                        P[L.klc_off() + q + 9 * e] += kl[q];
                    }
                    P[L.kcs_off() + 0 + 9 * e] += kc;
                    P[L.kcs_off() + 4 + 9 * e] += kc;
                    P[L.kcs_off() + 8 + 9 * e] += kc;
                }
            }
        } else {
            for (int e = warp; e < nE; e += nwarps) {
                const double ef = jb.ef[e];
                T ne = 0, ki[9], kl[9], kc = 0;
                CurvSum<T> a[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) { a[q].zero(); ki[q] = kl[q] = 0; }
                for (int n = lane; n < N; n += 32) {
                    const T f = fd_stat<T>(Es[n], ef, jb.T_kelvin);
                    ne += f;
                    kc += f * Cs[n];
#pragma unroll
                    for (int q = 0; q < 9; ++q) {
                        a[q].sub(curv, curvS, curvC, q * N + n, f);
                        ki[q] += icn[q * N + n] * f;
                        kl[q] += lcn[q * N + n] * f;
                    }
                }
                ne = warp_sum(ne);
                kc = warp_sum(kc);
#pragma unroll
                for (int q = 0; q < 9; ++q) { a[q].warp_reduce(); ki[q] = warp_sum(ki[q]); kl[q] = warp_sum(kl[q]); }
                if (lane == 0) {
                    P[L.ne_off() + e] += ne;
                    if (jb.do_ahc)
                        for (int q = 0; q < 9; ++q) P[L.ahc_off() + q + 9 * e] += a[q].value();
                    if (jb.do_kubo) {
                        for (int q = 0; q < 9; ++q) {
                            P[L.kic_off() + q + 9 * e] += ki[q];
                            P[L.klc_off() + q + 9 * e] += kl[q];
                        }
                        P[L.kcs_off() + 0 + 9 * e] += kc;
                        P[L.kcs_off() + 4 + 9 * e] += kc;
                        P[L.kcs_off() + 8 + 9 * e] += kc;
                    }
                }
            }
        }
    }
}

// Optical Hall tensors of one rank's k-points (the reference computes them
// with do_ahc, src/core.f90:221-230):
//   velo_ahc_tens (src/kubo.f90:86-140)
//       o(i,j,w,e) = sum_{n != m} (f(e,n) - f(e,m)) Im(c_nm) Wv_nm,
//       Wv_nm = 1 / ((E_n - E_m)^2 - (hw_w + i eta)^2)
//   kubo_ohc_tens (src/kubo.f90:146-198), no degeneracy guard (D9)
//       z(i,j,w,e) = sum_{n != m} g_nm (f(e,m) - f(e,n)),
//       g_nm = i c_nm / ((E_m - E_n)(E_m - E_n - hw_w - i eta))
// with c_nm(i,j) = V_i(n,m) V_j(m,n).  Both are regrouped by band,
//       o = sum_n f(e,n) Yv_n,  Yv_n = sum_m (Im c_nm - Im c_mn) Wv_nm   (Wv symmetric)
//       z = sum_n f(e,n) Yo_n,  Yo_n = sum_m (g_mn - g_nm),
// so a Fermi sweep costs N (n_eF + N) per photon energy instead of N^2 n_eF.
// The pair terms of two bands of equal occupation cancel in sum_n f Y_n only
// as far as Y_n is exact, so in the FP32 form the per-band sums and the
// contraction run in double-FP32 (TwoSum), as for the AHC curvature.  The
// energy differences are formed once per k in FP64 and kept as two T parts,
// so that (E_n - E_m) -+ hw cancels without loss near a resonance.
template <typename T>
__global__ void __launch_bounds__(256) opt_hall_kernel(DevModel md, JobDev jb, int64_t nk, const double* __restrict__ Eg,
                                                       const cplx<T>* __restrict__ Vg, const int* __restrict__ skip,
                                                       double* __restrict__ partials) {
    constexpr bool f32 = sizeof(T) == 4;
    constexpr int ET = f32 ? 64 : 8;   // Fermi energies per occupation tile
    extern __shared__ unsigned char smem_raw[];
    const int N = md.N, NN = N * N, ld = N + 1;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    cplx<T>* Vs = reinterpret_cast<cplx<T>*>(smem_raw);   // [3][N][ld]
    T* Ys = reinterpret_cast<T*>(Vs + 3 * N * ld);         // [N][36] per-band sums (leading part)
    T* Yc = Ys + N * 36;                                   // [N][36] remainders (FP32 form only)
    T* fs = f32 ? Yc + N * 36 : Yc;                        // [ET][N] occupations of one tile of Fermi energies
    T* dEh = fs + ET * N;                                  // FP32 form: [N][N] E_n - E_m, leading part
    T* dEl = dEh + NN;                                     //            and remainder
    T* part = dEl + NN;                                    //            [nwarps][32][36] lane terms
    __shared__ double Es[kMaxN];
    const AccLayout L{jb.nE, jb.nval, jb.nW};
    double* P = partials + (size_t)blockIdx.x * L.size();
    for (int64_t k = blockIdx.x; k < nk; k += gridDim.x) {
        if (skip && skip[k]) continue;
        __syncthreads();
        for (int e = tid; e < 3 * NN; e += nt) {
            const int a = e / NN, r = e % NN;
            Vs[(a * N + r / N) * ld + r % N] = Vg[(size_t)k * 3 * NN + e];
        }
        for (int n = tid; n < N; n += nt) Es[n] = Eg[(size_t)k * N + n];
        if constexpr (f32) {
            // E_n - E_m as an FP32 hi/lo pair from FP32 hi/lo energies (no FP64 per pair)
            __shared__ float s_Eh[kMaxN], s_El[kMaxN];
            __syncthreads();
            for (int n = tid; n < N; n += nt) {
                s_Eh[n] = (float)Es[n];
                s_El[n] = (float)(Es[n] - (double)s_Eh[n]);
            }
            __syncthreads();
            for (int e = tid; e < NN; e += nt) {
                const int n = e / N, m = e % N;
                float h, l;
                df_diff(s_Eh[n], s_El[n], s_Eh[m], s_El[m], h, l);
                dEh[e] = h;
                dEl[e] = l;
            }
        }
        for (int w = 0; w < jb.nW; ++w) {
            __syncthreads();
            const double hwd = jb.hw[w];
            const T hwh = (T)hwd, hwl = (T)(hwd - (double)hwh), eta = (T)jb.eta;
            // per-band sums Y_n: warp per band, lanes over m
            for (int n = warp; n < N; n += nwarps) {
                T acc[36];
#pragma unroll
                for (int q = 0; q < 36; ++q) acc[q] = (T)0;
                for (int m = lane; m < N; m += 32) {
                    if (m == n) continue;
                    T d, dm, dp;
                    if constexpr (f32) {
                        const T dh = dEh[n * N + m], dl = dEl[n * N + m];
                        d = dh + dl;
                        dm = ((dh - hwh) + dl) - hwl;
                        dp = ((dh + hwh) + dl) + hwl;
                    } else {
                        const double dd = Es[n] - Es[m];
                        d = dd;
                        dm = dd - hwd;
                        dp = dd + hwd;
                    }
                    // Wv = (ar + 2 i hw eta) / |A|^2,  A = (d - hw)(d + hw) + eta^2 - 2 i hw eta
                    const T ar = dm * dp + eta * eta, ai = (T)2 * hwh * eta;
                    const T an = (T)1 / (ar * ar + ai * ai);
                    const T wvr = ar * an, wvi = ai * an;
                    // g_nm = c_nm (B1i + i B1r) / |B1|^2,  B1 = d (d + hw) + i d eta
                    // g_mn = c_mn (B2i + i B2r) / |B2|^2,  B2 = d (d - hw) - i d eta
                    const T b1r = d * dp, b1i = d * eta, b2r = d * dm, b2i = -d * eta;
                    const T n1 = (T)1 / (b1r * b1r + b1i * b1i), n2 = (T)1 / (b2r * b2r + b2i * b2i);
                    const T g1r = b1i * n1, g1i = b1r * n1, g2r = b2i * n2, g2i = b2r * n2;
#pragma unroll
                    for (int j = 0; j < 3; ++j)
#pragma unroll
                        for (int i = 0; i < 3; ++i) {
                            const cplx<T> cnm = Vs[(i * N + n) * ld + m] * Vs[(j * N + m) * ld + n];
                            const cplx<T> cmn = Vs[(i * N + m) * ld + n] * Vs[(j * N + n) * ld + m];
                            const int q = 2 * (i + 3 * j);
                            const T dv = cnm.im - cmn.im;
                            acc[q] += dv * wvr;
                            acc[q + 1] += dv * wvi;
                            // g_mn - g_nm
                            acc[18 + q] += (cmn.re * g2r - cmn.im * g2i) - (cnm.re * g1r - cnm.im * g1i);
                            acc[18 + q + 1] += (cmn.re * g2i + cmn.im * g2r) - (cnm.re * g1i + cnm.im * g1r);
                        }
                }
                if constexpr (f32) {
                    T* pw = part + warp * 32 * 36;
#pragma unroll
                    for (int q = 0; q < 36; ++q) pw[lane * 36 + q] = acc[q];
                    __syncwarp();
                    for (int q = lane; q < 36; q += 32) {
                        DF r{0.f, 0.f};
                        for (int l = 0; l < 32; ++l) df_add(r, pw[l * 36 + q]);
                        Ys[n * 36 + q] = r.s;
                        Yc[n * 36 + q] = r.c;
                    }
                    __syncwarp();
                } else {
#pragma unroll
                    for (int q = 0; q < 36; ++q) {
                        const T v = warp_sum(acc[q]);
                        if (lane == 0) Ys[n * 36 + q] = v;
                    }
                }
            }
            // contraction with the occupations, tile by tile of Fermi energies
            for (int e0 = 0; e0 < jb.nE; e0 += ET) {
                const int ne = min(ET, jb.nE - e0);
                __syncthreads();
                for (int t = tid; t < ne * N; t += nt) {
                    const int e = t / N, n = t % N;
                    fs[e * N + n] = (T)fd_stat<double>(Es[n], jb.ef[e0 + e], jb.T_kelvin);
                }
                __syncthreads();
                for (int t = tid; t < ne * 36; t += nt) {
                    const int e = t / 36, q = t % 36;
                    double v;
                    if constexpr (f32) {
                        DF r{0.f, 0.f};
                        for (int n = 0; n < N; ++n) {
                            const float f = fs[e * N + n];
                            df_add_prod(r, Ys[n * 36 + q], f);
                            r.c = __fmaf_rn(Yc[n * 36 + q], f, r.c);
                        }
                        v = (double)r.s + (double)r.c;
                    } else {
                        v = 0.0;
                        for (int n = 0; n < N; ++n) v += Ys[n * 36 + q] * fs[e * N + n];
                    }
                    const int base = q < 18 ? L.vah_off() : L.koh_off();
                    P[base + (q % 18) + 18 * (w + jb.nW * (e0 + e))] += v;
                }
            }
        }
    }
}

__global__ void reduce_kernel(const double* __restrict__ partials, int n_cta, int size, double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < size; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < n_cta; ++c) s += partials[(size_t)c * size + i];
        out[i] = s;
    }
}

}  // namespace

int bandsum_ctas() {
    int dev = 0, sms = 148;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return 2 * sms;
}

template <typename T>
size_t bandsum_smem(int N, bool tables) {
    size_t b = 3 * (size_t)N * (N + 1) * sizeof(cplx<T>);
    b += (9 * (size_t)N + kMaxN) * sizeof(double);
    b += (18 * (size_t)N + 18 * kMaxN + kMaxN + (tables ? 2 * (size_t)N * (N + 1) : 0)) * sizeof(T);
    return (b + 15) & ~(size_t)15;
}

template <typename T>
cudaError_t launch_bandsum(const DevModel& m, const JobDev& j, int64_t nk, const double* E, const cplx<T>* V, const T* CSV,
                           const int* skip, double* partials, int n_cta, cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    const bool tables = bandsum_smem<T>(m.N, true) <= 227 * 1024;
    size_t smem = bandsum_smem<T>(m.N, tables);
    // the GEMM form of the IC contraction: FP32 form, N <= 32, with its W and G arrays
    const bool gemm = sizeof(T) == 4 && m.N <= 32 && tables;
    if (gemm)
        smem += 16 + (2 * 3 * 32 * 33 + 3 * kMaskCap) * sizeof(cplx<T>) + 32 * sizeof(T) + kMaskCap * sizeof(int) +
                32 * 32 * sizeof(short);
    auto go = [&](auto kern) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        kern<<<n_cta, 256, smem, s>>>(m, j, nk, E, V, CSV, skip, partials, tables ? 1 : 0);
        return cudaGetLastError();
    };
    if constexpr (sizeof(T) == 4) {
        if (gemm) return go(bandsum_kernel<T, true>);
    }
    return go(bandsum_kernel<T, false>);
}

// The FP32 form of opt_hall_kernel for N <= 32 and few (hbar omega, E_F) pairs:
// one k-point per warp, lane n = band n, the sum over m in registers (no
// shared-memory staging of V, no block barrier, no cross-lane reduction of the
// per-band sums).  V is Hermitian (to the bit: the gauge step forms it so), so
// lane n reads row n of V^i as the conjugate of column n, V^i(n, m) =
// conj(V^i(m, n)), one coalesced row m per step, and with c^ij = V^i_nm V^j_mn
// = v_i conj(v_j) the (m, n) products are conj(c^ij) and c^ji = conj(c^ij):
//     vah^ij += 2 Im(c^ij) Wv            (vah^ji = -vah^ij, vah^ii = 0)
//     koh^ij += c (g_mn) - c (g_nm) regrouped as (A + B, C - D), koh^ji = (A - B, C + D)
// with A = Re c (g2r - g1r), B = Im c (g2i + g1i), C = Re c (g2i - g1i),
// D = Im c (g2r + g1r): 24 double-FP32 sums per lane instead of 36.  The
// occupation contraction sum_n f_n Y_n is a double-FP32 butterfly across the
// lanes; each warp keeps its k-points' sums in shared memory and the CTA adds
// its warps' sums to its slice in a fixed order.
constexpr int OHW_WARPS = 8;
constexpr int OHW_MAX_PAIRS = 32;   // (hbar omega, E_F) pairs per launch in this form

__device__ __forceinline__ void ohw_df_warp_sum(float& s, float& c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_xor_sync(0xffffffffu, s, o), c2 = __shfl_xor_sync(0xffffffffu, c, o);
        const float t = s + s2, bb = t - s;
        const float e = (s - (t - bb)) + (s2 - bb);
        s = t;
        c = c + c2 + e;
    }
}

__global__ void __launch_bounds__(32 * OHW_WARPS, 2) opt_hall_warp_kernel(DevModel md, JobDev jb, int64_t nk,
                                                                      const double* __restrict__ Eg,
                                                                      const cplx<float>* __restrict__ Vg,
                                                                      const int* __restrict__ skip,
                                                                      double* __restrict__ partials) {
    extern __shared__ double ohw_acc[];   // [warp][(e * nW + w) * 36 + q]
    const int N = md.N, NN = N * N;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const unsigned FULL = 0xffffffffu;
    const int npair = jb.nW * jb.nE;
    double* Aw = ohw_acc + (size_t)wp * npair * 36;
    for (int i = lane; i < npair * 36; i += 32) Aw[i] = 0.0;
    __syncwarp();
    const float eta = (float)jb.eta;
    const bool act = lane < N;
    for (int64_t k = (int64_t)blockIdx.x * OHW_WARPS + wp; k < nk; k += (int64_t)gridDim.x * OHW_WARPS) {
        if (skip && skip[k]) continue;
        const double En = act ? Eg[(size_t)k * N + lane] : 0.0;
        const float eh = (float)En, el = (float)(En - (double)eh);
        const cplx<float>* Vk = Vg + (size_t)k * 3 * NN;
        for (int w = 0; w < jb.nW; ++w) {
            const double hwd = jb.hw[w];
            const float hwh = (float)hwd, hwl = (float)(hwd - (double)hwh);
            DF acc[24];
#pragma unroll
            for (int q = 0; q < 24; ++q) acc[q] = DF{0.f, 0.f};
            for (int m = 0; m < N; ++m) {
                cplx<float> v[3];
#pragma unroll
                for (int i = 0; i < 3; ++i) v[i] = act ? conjg(Vk[(size_t)(i * N + m) * N + lane]) : mk(0.f, 0.f);
                const float ehm = __shfl_sync(FULL, eh, m), elm = __shfl_sync(FULL, el, m);
                if (!act || m == lane) continue;
                float dh, dl;
                df_diff(eh, el, ehm, elm, dh, dl);
                const float d = dh + dl;
                const float dm = ((dh - hwh) + dl) - hwl;
                const float dp = ((dh + hwh) + dl) + hwl;
                const float ar = dm * dp + eta * eta, ai = 2.f * hwh * eta;
                const float an = 1.f / (ar * ar + ai * ai);
                const float wvr = ar * an, wvi = ai * an;
                const float b1r = d * dp, b1i = d * eta, b2r = d * dm, b2i = -d * eta;
                const float n1 = 1.f / (b1r * b1r + b1i * b1i), n2 = 1.f / (b2r * b2r + b2i * b2i);
                const float g1r = b1i * n1, g1i = b1r * n1, g2r = b2i * n2, g2i = b2r * n2;
                const float gar = g2r - g1r, gbi = g2i + g1i, gci = g2i - g1i, gdr = g2r + g1r;
#pragma unroll
                for (int pq = 0; pq < 3; ++pq) {
                    const int i = pq < 2 ? 0 : 1, j = pq == 0 ? 1 : 2;   // (x,y), (x,z), (y,z)
                    const float cr = v[i].re * v[j].re + v[i].im * v[j].im;
                    const float ci = v[i].im * v[j].re - v[i].re * v[j].im;
                    const float dv = 2.f * ci;
                    df_add(acc[6 * pq + 0], dv * wvr);
                    df_add(acc[6 * pq + 1], dv * wvi);
                    df_add(acc[6 * pq + 2], cr * gar);
                    df_add(acc[6 * pq + 3], ci * gbi);
                    df_add(acc[6 * pq + 4], cr * gci);
                    df_add(acc[6 * pq + 5], ci * gdr);
                }
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const float c = v[i].re * v[i].re + v[i].im * v[i].im;
                    df_add(acc[18 + 2 * i], c * gar);
                    df_add(acc[18 + 2 * i + 1], c * gci);
                }
            }
            for (int e = 0; e < jb.nE; ++e) {
                const float f = act ? (float)fd_stat<double>(En, jb.ef[e], jb.T_kelvin) : 0.f;
                double* A = Aw + (size_t)(e * jb.nW + w) * 36;
                // sum_n f_n Y_n[q] across the lanes, one value at a time
                auto lane_sum = [&](const DF& y) -> double {
                    const float p = f * y.s;
                    float rs = p, rc = fmaf(f, y.c, fmaf(f, y.s, -p));
                    ohw_df_warp_sum(rs, rc);
                    return (double)rs + (double)rc;
                };
#pragma unroll
                for (int pq = 0; pq < 3; ++pq) {
                    const int i = pq < 2 ? 0 : 1, j = pq == 0 ? 1 : 2;
                    const int qij = 2 * (i + 3 * j), qji = 2 * (j + 3 * i);
                    const double vr = lane_sum(acc[6 * pq + 0]), vi = lane_sum(acc[6 * pq + 1]);
                    const double ka = lane_sum(acc[6 * pq + 2]), kb = lane_sum(acc[6 * pq + 3]);
                    const double kc = lane_sum(acc[6 * pq + 4]), kd = lane_sum(acc[6 * pq + 5]);
                    if (lane == 0) {
                        A[qij] += vr;
                        A[qij + 1] += vi;
                        A[qji] -= vr;
                        A[qji + 1] -= vi;
                        A[18 + qij] += ka + kb;
                        A[18 + qij + 1] += kc - kd;
                        A[18 + qji] += ka - kb;
                        A[18 + qji + 1] += kc + kd;
                    }
                }
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int qii = 2 * (i + 3 * i);
                    const double ka = lane_sum(acc[18 + 2 * i]), kc = lane_sum(acc[18 + 2 * i + 1]);
                    if (lane == 0) {
                        A[18 + qii] += ka;
                        A[18 + qii + 1] += kc;
                    }
                }
                __syncwarp();
            }
        }
    }
    __syncthreads();
    // the CTA's slice: its warps' sums added in warp order
    const AccLayout L{jb.nE, jb.nval, jb.nW};
    double* P = partials + (size_t)blockIdx.x * L.size();
    for (int t = threadIdx.x; t < npair * 36; t += blockDim.x) {
        double v = 0.0;
        for (int u = 0; u < OHW_WARPS; ++u) v += ohw_acc[(size_t)u * npair * 36 + t];
        const int ew = t / 36, q = t % 36;   // ew = e * nW + w
        const int base = q < 18 ? L.vah_off() : L.koh_off();
        P[base + (q % 18) + 18 * ew] += v;
    }
}

template <typename T>
cudaError_t launch_opt_hall(const DevModel& m, const JobDev& j, int64_t nk, const double* E, const cplx<T>* V,
                            const int* skip, double* partials, int n_cta, cudaStream_t s) {
    if (nk <= 0 || j.nW <= 0) return cudaSuccess;
    if (sizeof(T) == 4 && m.N <= 32 && j.nW * j.nE <= OHW_MAX_PAIRS) {
        const size_t smem = (size_t)OHW_WARPS * j.nW * j.nE * 36 * sizeof(double);
        cudaError_t e = cudaFuncSetAttribute(opt_hall_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        opt_hall_warp_kernel<<<n_cta, 32 * OHW_WARPS, smem, s>>>(m, j, nk, E, reinterpret_cast<const cplx<float>*>(V),
                                                                  skip, partials);
        return cudaGetLastError();
    }
    const size_t N = m.N, ET = sizeof(T) == 4 ? 64 : 8;
    size_t smem = 3 * N * (N + 1) * sizeof(cplx<T>) + (N * 36 + ET * N) * sizeof(T);
    if (sizeof(T) == 4) smem += (N * 36 + 2 * N * N + 8 * 32 * 36) * sizeof(T);   // Yc, dEh, dEl, part
    cudaError_t e = cudaFuncSetAttribute(opt_hall_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(opt_hall_kernel<T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    opt_hall_kernel<T><<<n_cta, 256, smem, s>>>(m, j, nk, E, V, skip, partials);
    return cudaGetLastError();
}
template cudaError_t launch_opt_hall<double>(const DevModel&, const JobDev&, int64_t, const double*,
                                             const cplx<double>*, const int*, double*, int, cudaStream_t);
template cudaError_t launch_opt_hall<float>(const DevModel&, const JobDev&, int64_t, const double*,
                                            const cplx<float>*, const int*, double*, int, cudaStream_t);

// Per-k AHC integrand at one Fermi energy and the band gap there (inputs of
// the adaptive refinement).  out[pos][0..2] = the (y,z), (z,x), (x,y) entries
// of the term kubo_ahc_tens adds for this k (src/kubo.f90:37-78),
//     -sum_n f_n curv_n(i,j) = 2 sum_{n<m} (f_n - f_m) Im(V_i,nm V_j,mn) / (E_m - E_n)^2
// (the (n,m) and (m,n) terms of the reference's double sum are equal and
// opposite, so the pair form drops the occupied-occupied cancellation), and
// out[pos][3] = E_c - E_v across the Fermi energy (twice the distance to the
// nearest band when it lies outside all bands).  One warp per k-point.
template <typename T>
__global__ void __launch_bounds__(256) perk_kernel(int N, int64_t nk, const double* __restrict__ E,
                                                   const cplx<T>* __restrict__ V, double ef, double T_kelvin,
                                                   const int64_t* __restrict__ pos, int64_t pos0,
                                                   double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t k = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= nk) return;
    const double* Ek = E + (size_t)k * N;
    const size_t NN = (size_t)N * N;
    const cplx<T>* Vk = V + (size_t)k * 3 * NN;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int n = 0; n < N; ++n) {
        const double fn = fd_stat<double>(Ek[n], ef, T_kelvin);
        for (int m = n + 1 + lane; m < N; m += 32) {
            const double w = fn - fd_stat<double>(Ek[m], ef, T_kelvin);
            if (w == 0.0) continue;
            const double d = Ek[m] - Ek[n];
            const double c = 2.0 * w / (d * d);
            cplx<T> a[3], b[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                a[i] = Vk[i * NN + (size_t)n * N + m];
                b[i] = Vk[i * NN + (size_t)m * N + n];
            }
            // Im(V_i,nm V_j,mn) for (i,j) = (y,z), (z,x), (x,y)
            acc[0] += c * (double)(a[1] * b[2]).im;
            acc[1] += c * (double)(a[2] * b[0]).im;
            acc[2] += c * (double)(a[0] * b[1]).im;
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) acc[i] = warp_sum(acc[i]);
    if (lane == 0) {
        int nF = 0;
        while (nF < N && Ek[nF] < ef) ++nF;
        const double gap = nF == 0 ? 2.0 * (Ek[0] - ef) : nF == N ? 2.0 * (ef - Ek[N - 1]) : Ek[nF] - Ek[nF - 1];
        double* o = out + 4 * (size_t)(pos ? pos[k] : pos0 + k);
        o[0] = acc[0];
        o[1] = acc[1];
        o[2] = acc[2];
        o[3] = gap;
    }
}

template <typename T>
cudaError_t launch_perk(int N, int64_t nk, const double* E, const cplx<T>* V, double ef, double T_kelvin,
                        const int64_t* pos, int64_t pos0, double* out, cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    perk_kernel<T><<<(unsigned)((nk + 7) / 8), 256, 0, s>>>(N, nk, E, V, ef, T_kelvin, pos, pos0, out);
    return cudaGetLastError();
}
template cudaError_t launch_perk<double>(int, int64_t, const double*, const cplx<double>*, double, double,
                                         const int64_t*, int64_t, double*, cudaStream_t);
template cudaError_t launch_perk<float>(int, int64_t, const double*, const cplx<float>*, double, double,
                                        const int64_t*, int64_t, double*, cudaStream_t);

cudaError_t launch_reduce(const double* partials, int n_cta, int size, double* out, cudaStream_t s) {
    reduce_kernel<<<(size + 255) / 256, 256, 0, s>>>(partials, n_cta, size, out);
    return cudaGetLastError();
}

template cudaError_t launch_bandsum<double>(const DevModel&, const JobDev&, int64_t, const double*,
                                            const cplx<double>*, const double*, const int*, double*, int, cudaStream_t);
template cudaError_t launch_bandsum<float>(const DevModel&, const JobDev&, int64_t, const double*, const cplx<float>*,
                                           const float*, const int*, double*, int, cudaStream_t);

}  // namespace mepi

// ---------------------------------------------------------------------------
// Allocation-free variant of the band sums (mepi_bandsum_noalloc).
//
// Some callers of this library cannot allocate device memory at the moment
// they want the band sums: a host code that hands every byte of device memory
// to its own pool at start-up and forbids later allocations, a job confined to
// a fixed device-memory budget where a late cudaMalloc may fail, or a loop that
// cannot afford cudaMalloc's latency and implicit synchronisation.  For them
// this entry point keeps its only scratch -- the per-CTA FP64 partial sums --
// in a file-scope device array of fixed size instead of a cudaMalloc'd buffer;
// the caller passes device pointers for every input and output.
namespace mepi {
namespace {
constexpr size_t kNoAllocDoubles = size_t(1) << 19;  // 4 MiB of FP64 partial sums
constexpr int kNoAllocCtas = 152;                     // CTAs (slices) of the variant
constexpr int kMaxDevices = 64;
static __device__ __align__(256) double g_noalloc_partials[kNoAllocDoubles];

std::mutex g_noalloc_mu;
struct NoAllocSlot {
    unsigned long long ctx_id = 0;   // CUDA context the address belongs to
    double* ptr = nullptr;
};
NoAllocSlot g_noalloc_slot[kMaxDevices];

// Unique id of the calling thread's current CUDA context (cuCtxGetId through
// the runtime's driver entry point), 0 if it cannot be had.
unsigned long long current_ctx_id() {
    using GetCurrent = int (*)(void**);
    using GetId = int (*)(void*, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(p);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(p);
        looked_up = true;
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Device address of the scratch array on the current device.  The host-side
// symbol is only a stand-in, not a device address, so the address is looked
// up with cudaGetSymbolAddress once per device, with that device current, and
// looked up again when the device's context changes (after a cudaDeviceReset
// the module is loaded anew and the array may sit elsewhere).
cudaError_t noalloc_scratch(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocSlot& slot = g_noalloc_slot[dev];
    const unsigned long long id = current_ctx_id();   // 0 before the context exists
    if (!slot.ptr || id == 0 || id != slot.ctx_id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);   // initialises the context if needed
        if (e != cudaSuccess) return e;
        slot.ptr = static_cast<double*>(p);
        slot.ctx_id = current_ctx_id();
    }
    *out = slot.ptr;
    return cudaSuccess;
}
}  // namespace

}  // namespace mepi

extern "C" int mepi_bandsum_noalloc(int32_t n_wf, int64_t n_k, const double* en_k, const double* V,
                                    const double* csv, int32_t n_eF, const double* ef_lst, double T_kelvin,
                                    int32_t valence_bands, uint32_t outputs, double kubo_tol, double* sums,
                                    void* stream) {
    using namespace mepi;
    if (n_wf <= 0 || n_wf > kMaxN || n_k < 0 || n_eF <= 0 || valence_bands < 0 || valence_bands > n_wf)
        return MEPI_ERR_ARG;
    if (!ef_lst || !sums || (n_k > 0 && (!en_k || !V))) return MEPI_ERR_ARG;
    if (!(kubo_tol >= 0.0) || !std::isfinite(T_kelvin) || !std::isfinite(kubo_tol)) return MEPI_ERR_ARG;
    if (outputs & ~(uint32_t)(MEPI_OUT_AHC | MEPI_OUT_MEP_NIU | MEPI_OUT_KUBO_MEP)) return MEPI_ERR_ARG;
    // bound the slice size in 64-bit arithmetic before any int-sized layout
    const int64_t slice = 37 * (int64_t)n_eF + 27 * (int64_t)valence_bands;
    if (slice * kNoAllocCtas > (int64_t)kNoAllocDoubles) return MEPI_ERR_SCRATCH;
    const AccLayout L{n_eF, valence_bands};
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* scratch = nullptr;
    if (noalloc_scratch(&scratch) != cudaSuccess) return MEPI_ERR_CUDA;
    // the array keeps the previous call's sums: clear this call's slices
    if (cudaMemsetAsync(scratch, 0, (size_t)kNoAllocCtas * L.size() * sizeof(double), s) != cudaSuccess)
        return MEPI_ERR_CUDA;
    DevModel md{};
    md.N = n_wf;
    md.kubo_tol = kubo_tol;
    JobDev jb{};
    jb.nE = n_eF;
    jb.nval = valence_bands;
    jb.do_ahc = (outputs & MEPI_OUT_AHC) ? 1 : 0;
    jb.do_mep = (outputs & MEPI_OUT_MEP_NIU) ? 1 : 0;
    jb.do_kubo = (outputs & MEPI_OUT_KUBO_MEP) ? 1 : 0;
    jb.T_kelvin = T_kelvin;
    jb.ef = ef_lst;
    if (launch_bandsum<double>(md, jb, n_k, en_k, reinterpret_cast<const cplx<double>*>(V), csv, nullptr, scratch,
                               kNoAllocCtas, s) != cudaSuccess)
        return MEPI_ERR_CUDA;
    if (launch_reduce(scratch, kNoAllocCtas, L.size(), sums, s) != cudaSuccess) return MEPI_ERR_CUDA;
    return MEPI_OK;
}
