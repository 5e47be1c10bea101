// Internal declarations shared by the CUDA translation units of libmepi_gb300.
//
// Device data layout (C order, matrices row-major, element (n,m) at n*N+m):
//   S stack      S[R][pair][blk]        complex<double>, pair = n*N+m,
//                blk 0: H(R); 1..3: (C R)_a H(R); 4..6: r_a(R);
//                7..9: (C R)_a r_b(R) - (C R)_b r_a(R) for (a,b) = (x,y),(x,z),(y,z)
//                with C = a_latt (use_cart_velo) or 2*pi*I; 4 blocks without r(R).
//   W blocks     W[k][blk][n][m]        complex<T>, the Wannier-gauge H, H_a, A_a,
//                Omega_q per k-point after the tau phase epilogue.
//   E, U         E[k][n] ascending, U[k][i][n] = component i of eigenvector n;
//                the band kernels always read FP64 energies (E64 in the mixed
//                form, refined against the FP64 H64[k][n][m]).
//   HA           HA[k][6][n][m]          complex<T>: Hbar_a (a=0..2), Abar_a.
//   OD           OD[k][3][n]             complex<T>: diag(U^dag Omega_q U).
//   V            V[k][3][n][m]           complex<T>: velocity matrices.
//   CSV          CSV[k][n]               T: 0.5 Re(A_nn . om_vect_n) per band.
//   partials     per-CTA FP64 accumulators reduced in a fixed order.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mepi {

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kAuToEv = 27.211385;                    // src/constants.f90:19
constexpr double kKbEhK = 8.6173303e-5 / 27.211385;      // src/constants.f90:22
constexpr double kMinTemp = 1e-2;                        // src/statistics.f90:32
constexpr int kMaxN = 64;                                // largest n_wf supported

template <typename T> struct cplx { T re, im; };

// Division by a divisor fixed for the kernel (a band count N or N^2) by one
// multiply-high: q = umulhi(e, m), m = floor((2^32 - 1) / d) + 1 >= 2^32 / d,
// which is exact for every e with e d < 2^32 (the element indices here are
// below 6 N^2 with N <= 64).
struct FastDiv {
    uint32_t m, d;
    __host__ __device__ explicit FastDiv(int d_) : m(0xFFFFFFFFu / (uint32_t)d_ + 1u), d((uint32_t)d_) {}
    __device__ __forceinline__ int div(int e) const { return (int)__umulhi((uint32_t)e, m); }
    __device__ __forceinline__ int mod(int e) const { return e - div(e) * (int)d; }
};

template <typename T> __host__ __device__ __forceinline__ cplx<T> mk(T r, T i) { cplx<T> c; c.re = r; c.im = i; return c; }
template <typename T> __host__ __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return mk(a.re + b.re, a.im + b.im); }
template <typename T> __host__ __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return mk(a.re - b.re, a.im - b.im); }
template <typename T> __host__ __device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b) {
    return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> operator*(T s, cplx<T> a) { return mk(s * a.re, s * a.im); }
template <typename T> __host__ __device__ __forceinline__ cplx<T> conjg(cplx<T> a) { return mk(a.re, -a.im); }
// a * conj(b)
template <typename T> __host__ __device__ __forceinline__ cplx<T> mul_cj(cplx<T> a, cplx<T> b) {
    return mk(a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im);
}
// conj(a) * b
template <typename T> __host__ __device__ __forceinline__ cplx<T> cj_mul(cplx<T> a, cplx<T> b) {
    return mk(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}
// acc += a * b
template <typename T> __host__ __device__ __forceinline__ void fma_c(cplx<T>& acc, cplx<T> a, cplx<T> b) {
    acc.re = fma(a.re, b.re, acc.re); acc.re = fma(-a.im, b.im, acc.re);
    acc.im = fma(a.re, b.im, acc.im); acc.im = fma(a.im, b.re, acc.im);
}
// acc += conj(a) * b
template <typename T> __host__ __device__ __forceinline__ void fma_cjc(cplx<T>& acc, cplx<T> a, cplx<T> b) {
    acc.re = fma(a.re, b.re, acc.re); acc.re = fma(a.im, b.im, acc.re);
    acc.im = fma(a.re, b.im, acc.im); acc.im = fma(-a.im, b.re, acc.im);
}
template <typename T> __host__ __device__ __forceinline__ cplx<T> times_i(cplx<T> a) { return mk(-a.im, a.re); }
template <typename T> __host__ __device__ __forceinline__ T abs2(cplx<T> a) { return a.re * a.re + a.im * a.im; }

// C = op(A) B for N x N complex matrices in shared memory (row stride ld),
// op(A) = A (adjA = false) or A^dag (adjA = true).  Each thread computes a
// 4 x 1 output tile (four rows, one column): with N = 32 a warp shares its four
// rows, so its A loads are broadcasts, and walks 32 consecutive columns of B,
// so no load of the warp meets a bank conflict; every B load feeds four
// complex multiply-adds.  Only i, j < N are read and written.  The caller
// synchronises before and after.
template <typename T, bool adjA>
__device__ __forceinline__ void smem_cgemm(int N, int ld, const cplx<T>* __restrict__ A, const cplx<T>* __restrict__ B,
                                           cplx<T>* __restrict__ Cm, int tid, int nt) {
    const int nrb = (N + 3) >> 2;
    for (int t = tid; t < nrb * N; t += nt) {
        const int rb = t / N, j = t - rb * N, r0 = 4 * rb;
        cplx<T> c[4];
#pragma unroll
        for (int x = 0; x < 4; ++x) c[x] = mk((T)0, (T)0);
        for (int l = 0; l < N; ++l) {
            const cplx<T> b = B[l * ld + j];
#pragma unroll
            for (int x = 0; x < 4; ++x) {
                const int r = r0 + x;
                if (r < N) fma_c(c[x], adjA ? conjg(A[l * ld + r]) : A[r * ld + l], b);
            }
        }
#pragma unroll
        for (int x = 0; x < 4; ++x)
            if (r0 + x < N) Cm[(r0 + x) * ld + j] = c[x];
    }
}

// Asynchronous prefetch of [p, p + bytes) into L2 (cp.async.bulk.prefetch.L2;
// nothing to wait for).  Issued only for a 16-byte aligned start and a whole
// number of 16-byte units inside the caller's buffer; otherwise a no-op.
__device__ __forceinline__ void l2_prefetch(const void* p, uint32_t bytes) {
    if ((reinterpret_cast<uintptr_t>(p) & 15u) != 0 || (bytes & 15u) != 0 || bytes == 0) return;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Upper-triangle element u (row-major over n <= m) -> (n, m).  Row n holds
// N - n elements and starts at off(n) = n (2N - n + 1) / 2.
__device__ __forceinline__ void upper_pair(int u, int N, int& n, int& mm) {
    const float b = 2.f * N + 1.f;
    int r = (int)((b - sqrtf(b * b - 8.f * u)) * 0.5f);
    r = r < 0 ? 0 : (r > N - 1 ? N - 1 : r);
    while (r > 0 && r * (2 * N - r + 1) / 2 > u) --r;
    while (r < N - 1 && (r + 1) * (2 * N - r) / 2 <= u) ++r;
    n = r;
    mm = r + (u - r * (2 * N - r + 1) / 2);
}

// C = A^dag B known to be Hermitian (A, B complex Np x Np in shared memory,
// row stride ld, Np even): only the 2 x 2 tiles on or above the diagonal are
// formed, walked compactly so that whole warps drop out, and the strictly
// upper elements are mirrored.
template <typename T>
__device__ __forceinline__ void smem_cgemm_herm(int Np, int ld, const cplx<T>* __restrict__ A,
                                                const cplx<T>* __restrict__ B, cplx<T>* __restrict__ Cm, int tid,
                                                int nt) {
    const int h = Np >> 1;
    for (int u = tid; u < h * (h + 1) / 2; u += nt) {
        int a, b;
        upper_pair(u, h, a, b);
        const int i0 = 2 * a, j0 = 2 * b;
        cplx<T> c00 = mk((T)0, (T)0), c01 = c00, c10 = c00, c11 = c00;
        for (int l = 0; l < Np; ++l) {
            const cplx<T> a0 = conjg(A[l * ld + i0]), a1 = conjg(A[l * ld + i0 + 1]);
            const cplx<T> b0 = B[l * ld + j0], b1 = B[l * ld + j0 + 1];
            fma_c(c00, a0, b0);
            fma_c(c01, a0, b1);
            fma_c(c10, a1, b0);
            fma_c(c11, a1, b1);
        }
        Cm[i0 * ld + j0] = c00;
        Cm[i0 * ld + j0 + 1] = c01;
        Cm[(i0 + 1) * ld + j0 + 1] = c11;
        if (i0 == j0) {
            Cm[(i0 + 1) * ld + j0] = conjg(c01);
        } else {
            Cm[(i0 + 1) * ld + j0] = c10;
            Cm[j0 * ld + i0] = conjg(c00);
            Cm[(j0 + 1) * ld + i0] = conjg(c01);
            Cm[j0 * ld + i0 + 1] = conjg(c10);
            Cm[(j0 + 1) * ld + i0 + 1] = conjg(c11);
        }
    }
}

// Compensated FP32 arithmetic (Knuth's TwoSum, TwoProduct by FMA, and the
// Dot2 summation of Ogita, Rump and Oishi, SIAM J. Sci. Comput. 26 (2005)):
// a dot product of FP32 numbers accumulated as an unevaluated sum s + c, as if
// in twice the working precision.  The _rn intrinsics are never contracted
// into FMAs, which the error-free transformations rely on.
struct DF {
    float s, c;
};
// acc += x (TwoSum: the rounding error of the leading sum goes to acc.c)
__device__ __forceinline__ void df_add(DF& acc, float x) {
    const float t = __fadd_rn(acc.s, x);
    const float bp = __fsub_rn(t, acc.s);
    const float e = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(t, bp)), __fsub_rn(x, bp));
    acc.s = t;
    acc.c = __fadd_rn(acc.c, e);
}
// (ah + al) - (bh + bl) as a normalised FP32 pair (h, l): TwoSum of the
// leading parts plus the difference of the remainders, about 2^-48 of the
// operands -- the FP64 difference of two FP64 energies split into hi + lo,
// without FP64 arithmetic
__device__ __forceinline__ void df_diff(float ah, float al, float bh, float bl, float& h, float& l) {
    const float s = __fsub_rn(ah, bh);
    const float bp = __fsub_rn(s, ah);
    const float t = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bp)), __fsub_rn(-bh, bp));
    const float lo = __fadd_rn(t, __fsub_rn(al, bl));
    h = __fadd_rn(s, lo);
    l = __fsub_rn(lo, __fsub_rn(h, s));
}
// a + b of two unevaluated sums
__device__ __forceinline__ DF df_sum(DF a, DF b) {
    DF r{a.s, __fadd_rn(a.c, b.c)};
    df_add(r, b.s);
    return r;
}
// sum over the 32 lanes of a warp, in double-FP32
__device__ __forceinline__ DF df_warp_sum(DF v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const DF w{__shfl_xor_sync(0xffffffffu, v.s, o), __shfl_xor_sync(0xffffffffu, v.c, o)};
        v = df_sum(v, w);
    }
    return v;
}
__device__ __forceinline__ void df_add_prod(DF& acc, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);          // a b = p + pe exactly
    const float t = __fadd_rn(acc.s, p);
    const float bp = __fsub_rn(t, acc.s);
    const float e = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(t, bp)), __fsub_rn(p, bp));  // acc.s + p = t + e
    acc.s = t;
    acc.c = __fadd_rn(acc.c, __fadd_rn(e, pe));
}

// C = op(A) B for complex FP32 Np x Np matrices in shared memory (row stride
// ld, Np even), accumulated in Dot2 so that the result is as if formed in
// twice the working precision; 2 x 2 output tiles per thread.  op(A) = A^dag
// when adjA.  Blo (optional) is a low-order part of B, added in plain FP32.
// Chi receives the rounded result; Clo (optional) the remainder
// (C = Chi + Clo to about 2^-44 relative).  With upper, only the tiles on or
// above the diagonal are formed (walked compactly, so that whole warps drop
// out) and the Hermitian mirror of the strictly upper elements is written (for
// products known to be Hermitian).
template <bool adjA>
__device__ __forceinline__ void cgemm_dot2(int Np, int ld, const cplx<float>* __restrict__ A,
                                           const cplx<float>* __restrict__ B, const cplx<float>* __restrict__ Blo,
                                           cplx<float>* __restrict__ Chi, cplx<float>* __restrict__ Clo, bool upper,
                                           int tid, int nt) {
    const int h = Np >> 1;
    const int ntile = upper ? h * (h + 1) / 2 : h * h;
    for (int t = tid; t < ntile; t += nt) {
        int a, b;
        if (upper) upper_pair(t, h, a, b);
        else { a = t / h; b = t % h; }
        const int i0 = 2 * a, j0 = 2 * b;
        DF re[2][2], im[2][2];
        cplx<float> lo[2][2];
#pragma unroll
        for (int x = 0; x < 2; ++x)
#pragma unroll
            for (int y = 0; y < 2; ++y) {
                re[x][y] = DF{0.f, 0.f};
                im[x][y] = DF{0.f, 0.f};
                lo[x][y] = mk(0.f, 0.f);
            }
        for (int l = 0; l < Np; ++l) {
            cplx<float> a[2];
            if (adjA) {
                a[0] = conjg(A[l * ld + i0]);
                a[1] = conjg(A[l * ld + i0 + 1]);
            } else {
                a[0] = A[i0 * ld + l];
                a[1] = A[(i0 + 1) * ld + l];
            }
            const cplx<float> b[2] = {B[l * ld + j0], B[l * ld + j0 + 1]};
#pragma unroll
            for (int x = 0; x < 2; ++x)
#pragma unroll
                for (int y = 0; y < 2; ++y) {
                    df_add_prod(re[x][y], a[x].re, b[y].re);
                    df_add_prod(re[x][y], -a[x].im, b[y].im);
                    df_add_prod(im[x][y], a[x].re, b[y].im);
                    df_add_prod(im[x][y], a[x].im, b[y].re);
                }
            if (Blo) {
                const cplx<float> bl[2] = {Blo[l * ld + j0], Blo[l * ld + j0 + 1]};
#pragma unroll
                for (int x = 0; x < 2; ++x)
#pragma unroll
                    for (int y = 0; y < 2; ++y) fma_c(lo[x][y], a[x], bl[y]);
            }
        }
#pragma unroll
        for (int x = 0; x < 2; ++x)
#pragma unroll
            for (int y = 0; y < 2; ++y) {
                const int r = i0 + x, c = j0 + y;
                const float cr = __fadd_rn(re[x][y].c, lo[x][y].re), ci = __fadd_rn(im[x][y].c, lo[x][y].im);
                const float hr = __fadd_rn(re[x][y].s, cr), hi = __fadd_rn(im[x][y].s, ci);
                if (upper && r > c) continue;   // the lower element of a diagonal tile comes from the mirror
                Chi[r * ld + c] = mk(hr, hi);
                if (Clo) Clo[r * ld + c] = mk(__fadd_rn(__fsub_rn(re[x][y].s, hr), cr), __fadd_rn(__fsub_rn(im[x][y].s, hi), ci));
                if (upper && r < c) Chi[c * ld + r] = mk(hr, -hi);
            }
    }
}

// Which k-points a launch covers: k = list ? list[i] : k_begin + i * k_stride.
struct KRange {
    int64_t k_begin, k_stride, count;
    const int64_t* list;     // device pointer or nullptr
    const double* kpts;      // device (count, 3) explicit k-points, or nullptr
    int32_t mp[3];
};

__device__ __forceinline__ int64_t k_of(const KRange& kr, int64_t i) {
    return kr.list ? kr.list[i] : kr.k_begin + i * kr.k_stride;
}

// Monkhorst-Pack point, src/k_space.f90:351-375 (kx fastest, 1-based q).
__device__ __forceinline__ void mp_kpt(const int32_t mp[3], int64_t ki, double k[3]) {
    int64_t q0 = ki % mp[0] + 1;
    int64_t q1 = (ki / mp[0]) % mp[1] + 1;
    int64_t q2 = ki / ((int64_t)mp[0] * mp[1]) + 1;
    k[0] = (2.0 * (double)q0 - (double)mp[0] - 1.0) / (2.0 * (double)mp[0]);
    k[1] = (2.0 * (double)q1 - (double)mp[1] - 1.0) / (2.0 * (double)mp[1]);
    k[2] = (2.0 * (double)q2 - (double)mp[2] - 1.0) / (2.0 * (double)mp[2]);
}

// Model constants the epilogues need, in constant-size device structs.
struct DevModel {
    int N, nR, nb;            // n_wf, n_R, stack blocks (10 with r(R), 4 without)
    int has_r, has_tau, semantics, do_gauge;
    double kubo_tol;
    double C[9];              // derivative weight matrix, row-major C[a*3+j]
    const cplx<double>* S;    // S stack (nR, N*N, nb)
    const double* R;          // R_frac (nR, 3)
    const double* tau;        // (N, 3) or nullptr
};

// Tight-binding phase epilogue of the Fourier sums for one (n,m) pair of one
// k-point, in arithmetic TE: from the raw sums X_b = sum_R exp(2 pi i k.R) S_b(R)
// it writes the W-gauge blocks, with psi = exp(2 pi i k.(tau_m - tau_n)) and
// dt = C (tau_m - tau_n):
//     H = psi X_0,  H_a = i (psi X_a + dt_a H),  A_b = psi X_{3+b},
//     Om_ab = i (psi X_Q + dt_a A_b - dt_b A_a)
// (the per-element angle 2 pi k.(R + tau_m - tau_n) of
// src/wann_interp.f90:192-281 factorised; the Wannier convention is tau = 0).
template <typename T, typename TE, int NB>
__device__ __forceinline__ void tb_epilogue(const DevModel& m, cplx<TE> psi, int pair, const cplx<TE> (&X)[NB],
                                            cplx<T>* __restrict__ Wk, int NN) {
    TE dt[3] = {(TE)0, (TE)0, (TE)0};
    if (m.has_tau) {
        const int n = pair / m.N, mm = pair % m.N;
        double d[3];
        for (int i = 0; i < 3; ++i) d[i] = m.tau[mm * 3 + i] - m.tau[n * 3 + i];
        for (int a = 0; a < 3; ++a) dt[a] = (TE)(m.C[a * 3 + 0] * d[0] + m.C[a * 3 + 1] * d[1] + m.C[a * 3 + 2] * d[2]);
    }
    const cplx<TE> H = psi * X[0];
    Wk[pair] = mk((T)H.re, (T)H.im);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const cplx<TE> v = times_i(psi * X[1 + a] + dt[a] * H);
        Wk[(size_t)(1 + a) * NN + pair] = mk((T)v.re, (T)v.im);
    }
    if constexpr (NB == 10) {
        cplx<TE> A[3];
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            A[b] = psi * X[4 + b];
            Wk[(size_t)(4 + b) * NN + pair] = mk((T)A[b].re, (T)A[b].im);
        }
        const int qa[3] = {0, 0, 1}, qb[3] = {1, 2, 2};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const cplx<TE> v = times_i(psi * X[7 + q] + dt[qa[q]] * A[qb[q]] - dt[qb[q]] * A[qa[q]]);
            Wk[(size_t)(7 + q) * NN + pair] = mk((T)v.re, (T)v.im);
        }
    }
}

// The same with psi from the k-point itself (one sincospi per element).
template <typename T, int NB>
__device__ __forceinline__ void ft_epilogue(const DevModel& m, const double k[3], int pair, const cplx<double> (&X)[NB],
                                            cplx<T>* __restrict__ Wk, int NN) {
    cplx<double> psi = mk(1.0, 0.0);
    if (m.has_tau) {
        const int n = pair / m.N, mm = pair % m.N;
        double x = 0.0;
        for (int i = 0; i < 3; ++i) x += k[i] * (m.tau[mm * 3 + i] - m.tau[n * 3 + i]);
        double s, c;
        sincospi(2.0 * x, &s, &c);
        psi = mk(c, s);
    }
    tb_epilogue<T, double, NB>(m, psi, pair, X, Wk, NN);
}


struct JobDev {
    int nE, nval, do_ahc, do_mep, do_kubo;
    double T_kelvin;
    const double* ef;         // device (nE)
    int nW = 0;               // photon energies of the optical Hall tensors (0 = off)
    const double* hw = nullptr;   // device (nW)
    double eta = 0.0;
};

// Layout of one CTA's FP64 accumulator slice.
struct AccLayout {
    int nE, nval, nW = 0;
    __host__ __device__ int ne_off() const { return 0; }
    __host__ __device__ int ahc_off() const { return nE; }
    __host__ __device__ int kic_off() const { return nE + 9 * nE; }
    __host__ __device__ int klc_off() const { return nE + 18 * nE; }
    __host__ __device__ int kcs_off() const { return nE + 27 * nE; }
    __host__ __device__ int mic_off() const { return nE + 36 * nE; }
    __host__ __device__ int mlc_off() const { return nE + 36 * nE + 9 * nval; }
    __host__ __device__ int mcs_off() const { return nE + 36 * nE + 18 * nval; }
    // velo_ahc and kubo_ohc: (3,3,nW,nE) complex as (re, im) pairs
    __host__ __device__ int vah_off() const { return nE + 36 * nE + 27 * nval; }
    __host__ __device__ int koh_off() const { return vah_off() + 18 * nW * nE; }
    __host__ __device__ int size() const { return nE + 36 * nE + 27 * nval + 36 * nW * nE; }
};

// ---- host launchers (one per translation unit) ----
template <typename T>
cudaError_t launch_ft_simt(const DevModel& m, const KRange& kr, cplx<T>* W, cudaStream_t s);
template <typename T>
cudaError_t launch_eig(int N, int64_t nk, const cplx<T>* W, int nbW, const float4* Hdf, T* E, cplx<T>* U,
                       int max_sweeps, int* sweeps_max, int* flag_cap, double degen_gap, int* redo_flag,
                       cudaStream_t s, int threads = 0, int kblock = 0, float gap_theta = 0.f,
                       bool warp_form = false);
// The mixed form's FP64-accurate H(k), upper triangle, as double-FP32 pairs: per
// element float4 (re_hi, im_hi, re_lo, im_lo), hi = the value rounded to FP32,
// lo = the rest rounded to FP32 (about 2^-48 relative).
cudaError_t launch_ft_h64(const DevModel& m, const KRange& kr, float4* Hdf, cudaStream_t s);
cudaError_t launch_refine(int N, int64_t nk, const float4* Hdf, const float* lam, cplx<float>* U, cplx<float>* Ulo, double* E64,
                          double degen_gap, int* redo_flag, cudaStream_t s);
template <typename T>
cudaError_t launch_rot(const DevModel& m, int64_t nk, const cplx<T>* W, const cplx<T>* U, cplx<T>* HA,
                       cplx<T>* OD, cudaStream_t s);
// tensor-core rotation of the mixed form (rot_tc.cu): n_wf <= 32 with the gauge transformation
bool rot_tc_supported(const DevModel& m);
cudaError_t launch_rot_tc(const DevModel& m, int64_t nk, const cplx<float>* W, const cplx<float>* U,
                          const cplx<float>* Ulo, cplx<float>* HA, cplx<float>* OD, int* err, cudaStream_t s);
template <typename T>
cudaError_t launch_gauge(const DevModel& m, int64_t nk, const double* E, const cplx<T>* HA, const cplx<T>* OD,
                         cplx<T>* V, T* CSV, cplx<T>* ODH, cudaStream_t s);
template <typename T>
cudaError_t launch_bandsum(const DevModel& m, const JobDev& j, int64_t nk, const double* E, const cplx<T>* V,
                           const T* CSV, const int* skip, double* partials, int n_cta, cudaStream_t s);
cudaError_t launch_reduce(const double* partials, int n_cta, int size, double* out, cudaStream_t s);
// per-k AHC integrand and gap at one Fermi energy into out[pos][4] (pos null: pos0 + k)
template <typename T>
cudaError_t launch_perk(int N, int64_t nk, const double* E, const cplx<T>* V, double ef, double T_kelvin,
                        const int64_t* pos, int64_t pos0, double* out, cudaStream_t s);
template <typename T>
cudaError_t launch_opt_hall(const DevModel& m, const JobDev& j, int64_t nk, const double* E, const cplx<T>* V,
                            const int* skip, double* partials, int n_cta, cudaStream_t s);

// Separable Fourier sums on a Monkhorst-Pack mesh (ft_sep.cu).  The R box
// stays resident; the slabs G2[qx][qy][iz][blk][pair] cover nqx consecutive qx
// (the whole mesh when they fit in the memory budget, else one slab after the
// other during the run).
struct SepPlan {
    bool ready = false;
    bool fp64 = false;              // built for the FP64 form (no FP32 slabs)
    int N = 0, nbk = 0, nbd = 0;    // n_wf, stack blocks, blocks in G2d (nbk, or 1 = H alone)
    int mp[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, nb[3] = {0, 0, 0};  // mesh, R box origin and size
    int nqx = 0;                    // qx per slab
    int built_qx0 = -1;             // first qx of the slab the arrays hold
    cplx<double>* box = nullptr;    // the stack on the R box, [ix][iy][iz][blk][pair]
    cplx<double>* G1 = nullptr;     // [qx][iy][iz][blk][pair] of one slab
    cplx<double>* G2d = nullptr;
    cplx<float>* G2f = nullptr;
    const double* tau = nullptr;
    size_t h2d_bytes = 0;
    size_t dev_bytes = 0;           // device memory the plan holds
    bool whole() const { return nqx == mp[0]; }
};
// 0: plan ready; 1: the model or mesh has no separable form here (non-integer
// R, an R box wider than 32, or not even one qx slab within the budget);
// 2/3: CUDA error / out of memory (the MEPI_ERR_* values).  budget 0 = half the
// free device memory.
int sep_plan_build(SepPlan& p, const DevModel& m, const double* R_host, const cplx<double>* S_host, const int mp[3],
                   bool fp64, size_t budget, cudaStream_t s);
// device bytes of the whole-mesh plan (0: no separable form for this model)
size_t sep_plan_want(const DevModel& m, const double* R_host, const int mp[3], bool fp64);
// enqueue the build of the slab that starts at qx0 (stream work only)
cudaError_t launch_sep_slab(SepPlan& p, int qx0, cudaStream_t s);
void sep_plan_free(SepPlan& p);
cudaError_t launch_sep_h64(const SepPlan& p, const KRange& kr, float4* Hdf, cudaStream_t s);
template <typename T>
cudaError_t launch_sep_w(const SepPlan& p, const DevModel& m, const KRange& kr, cplx<T>* W, cudaStream_t s);
int bandsum_ctas();

}  // namespace mepi
