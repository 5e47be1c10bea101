// Fourier sums of FT_R_to_k (src/wann_interp.f90:151-384) on a Monkhorst-Pack
// mesh by separable sums.
//
// For integer lattice vectors R inside a box [Rx0, Rx1] x [Ry0, Ry1] x
// [Rz0, Rz1] (missing R count as zero blocks) and MP points
// k_d = (2 q_d - n_d - 1) / (2 n_d), the phase exp(2 pi i k.R) factorises per
// axis, so every stack block S_b(R) (H, C R H, r, the curvature combinations)
// is summed as
//     G1[qx][Ry][Rz] = sum_Rx exp(2 pi i kx Rx) S(Rx, Ry, Rz)        (once per run)
//     G2[qx][qy][Rz] = sum_Ry exp(2 pi i ky Ry) G1[qx][Ry][Rz]      (once per run)
//     X(k)           = sum_Rz exp(2 pi i kz Rz) G2[qx][qy][Rz]      (per k)
// followed by the tight-binding phase epilogue.  The per-k stage costs nbz
// complex multiply-adds per element instead of nR, and the k-points of one
// (qx, qy) column share one G2 slab, so with the k-points ordered column by
// column the slab is read from HBM once and from L2 by the rest of the column.
//
// Precision: the FP64 form's plan is built in FP64 and keeps G2 in FP64 for all
// blocks.  The mixed form's plan sums over Rx in FP64 and over Ry in
// double-FP32 (about 2^-46 relative, off the 1/64-rate FP64 pipe).  The mixed
// form keeps all blocks in FP32 (nbz-term sums of FP32 values, about 1e-7
// relative) for its per-k work, plus FP64 slabs for the FP64-accurate H(k) of
// the eigenpair refinement (summed in double-FP32) and for its FP64 reruns (all
// blocks when they fit in memory, else H alone).
#include <algorithm>
#include <cmath>
#include <vector>

#include "mepi_internal.cuh"

namespace mepi {

namespace {

__device__ __forceinline__ double mp_coord(int q, int n) {  // 0-based q
    return (2.0 * (double)(q + 1) - (double)n - 1.0) / (2.0 * (double)n);
}

__device__ __forceinline__ cplx<double> phase(double k, int R) {
    double s, c;
    sincospi(2.0 * k * (double)R, &s, &c);
    return mk(c, s);
}

// G1[qx][iy][iz][e] = sum_ix phase(kx, Rx0 + ix) box[ix][iy][iz][e],  e = blk * NN + pair,
// for the qx of one slab [qx0, qx0 + gridDim.z)
// With df_out (the mixed form's plans) G1 is written as double-FP32 pairs,
// float4 (re_hi, im_hi, re_lo, im_lo) in the same 16 bytes, for sep_stage_b_df.
__global__ void sep_stage_a(const cplx<double>* __restrict__ box, cplx<double>* __restrict__ G1, int EL, int nbx,
                            int nby, int nbz, int rx0, int n1, int qx0, bool df_out) {
    const int yz = blockIdx.y, qx = blockIdx.z;   // qx relative to the slab's first qx0
    __shared__ cplx<double> ph[32];
    if (threadIdx.x < nbx) ph[threadIdx.x] = phase(mp_coord(qx0 + qx, n1), rx0 + (int)threadIdx.x);
    __syncthreads();
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < EL; e += gridDim.x * blockDim.x) {
        cplx<double> acc = mk(0.0, 0.0);
        for (int ix = 0; ix < nbx; ++ix) fma_c(acc, ph[ix], box[((size_t)ix * nby * nbz + yz) * EL + e]);
        const size_t o = ((size_t)qx * nby * nbz + yz) * EL + e;
        if (df_out) {
            const float hr = (float)acc.re, hi = (float)acc.im;
            reinterpret_cast<float4*>(G1)[o] = make_float4(hr, hi, (float)(acc.re - (double)hr), (float)(acc.im - (double)hi));
        } else {
            G1[o] = acc;
        }
    }
}

// G2[qx][qy][iz][e] = sum_iy phase(ky, Ry0 + iy) G1[qx][iy][iz][e] (qx within the
// slab); the first nbd blocks go to G2d (FP64), all blocks to G2f (FP32) when
// it is allocated.
__global__ void sep_stage_b(const cplx<double>* __restrict__ G1, cplx<double>* __restrict__ G2d,
                            cplx<float>* __restrict__ G2f, int NN, int nbk, int nbd, int nby, int nbz, int ry0, int n1,
                            int n2) {
    const int iz = blockIdx.y % nbz, qy = blockIdx.y / nbz, qx = blockIdx.z;
    __shared__ cplx<double> ph[32];
    if (threadIdx.x < nby) ph[threadIdx.x] = phase(mp_coord(qy, n2), ry0 + (int)threadIdx.x);
    __syncthreads();
    const int EL = nbk * NN;
    const size_t cell = ((size_t)qx * n2 + qy) * nbz + iz;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < EL; e += gridDim.x * blockDim.x) {
        cplx<double> acc = mk(0.0, 0.0);
        for (int iy = 0; iy < nby; ++iy) fma_c(acc, ph[iy], G1[(((size_t)qx * nby + iy) * nbz + iz) * EL + e]);
        if (e < nbd * NN) G2d[cell * nbd * NN + e] = acc;
        if (G2f) G2f[cell * EL + e] = mk((float)acc.re, (float)acc.im);
    }
}

__device__ __forceinline__ void item_coords(const KRange& kr, int64_t i, int q[3], double k[3]) {
    const int64_t ki = k_of(kr, i);
    q[0] = (int)(ki % kr.mp[0]);
    q[1] = (int)((ki / kr.mp[0]) % kr.mp[1]);
    q[2] = (int)(ki / ((int64_t)kr.mp[0] * kr.mp[1]));
    for (int a = 0; a < 3; ++a) k[a] = mp_coord(q[a], kr.mp[a]);
}

// Per-CTA item header: k, kz phases and slab offset of KI consecutive items,
// and whether they all lie in one (qx, qy) column (then each slab element is
// loaded once and applied to all KI items).
template <typename TG, int KI>
struct ItemHead {
    cplx<TG> ph[KI][32];
    cplx<TG> phi[KI][kMaxN];   // exp(2 pi i k.tau_n); psi_nm = conj(phi_n) phi_m
    double k[KI][3];
    size_t slab[KI];
    int n_items;
    int uniform;
};

template <typename TG, int KI>
__device__ void load_items(ItemHead<TG, KI>& h, const KRange& kr, int nbz, int rz0, size_t slab_elems,
                           const double* __restrict__ tau, int N, int qx0, int nqx) {
    const int64_t i0 = (int64_t)blockIdx.x * KI;
    if (threadIdx.x == 0) h.n_items = (int)(kr.count - i0 < KI ? kr.count - i0 : KI);
    if (threadIdx.x < KI) {
        const int it = threadIdx.x;
        int q[3] = {0, 0, 0};
        double k[3] = {0.0, 0.0, 0.0};
        if (i0 + it < kr.count) item_coords(kr, i0 + it, q, k);
        h.k[it][0] = k[0]; h.k[it][1] = k[1]; h.k[it][2] = k[2];
        // the caller keeps every item inside the resident slab [qx0, qx0 + nqx);
        // an item outside it is clamped to the slab rather than read out of bounds
        int rq = q[0] - qx0;
        rq = rq < 0 ? 0 : (rq >= nqx ? nqx - 1 : rq);
        h.slab[it] = ((size_t)rq * kr.mp[1] + q[1]) * slab_elems;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int u = 1;
        for (int it = 1; it < h.n_items; ++it) u &= (h.slab[it] == h.slab[0]) ? 1 : 0;
        h.uniform = u;
    }
    // phases in FP64 (rounded once to TG): formed once per CTA of KI items
    for (int e = threadIdx.x; e < KI * 32; e += blockDim.x) {
        const int it = e / 32, iz = e % 32;
        const cplx<double> p = iz < nbz ? phase(h.k[it][2], rz0 + iz) : mk(0.0, 0.0);
        h.ph[it][iz] = mk((TG)p.re, (TG)p.im);
    }
    if (tau)
        for (int e = threadIdx.x; e < KI * N; e += blockDim.x) {
            const int it = e / N, n = e % N;
            double sn, cs;
            sincospi(2.0 * (h.k[it][0] * tau[3 * n] + h.k[it][1] * tau[3 * n + 1] + h.k[it][2] * tau[3 * n + 2]), &sn,
                     &cs);
            h.phi[it][n] = mk((TG)cs, (TG)sn);
        }
    __syncthreads();
}

// acc[it] = sum_iz ph[it][iz] g[slab(it) + iz * zstride]
template <typename TG, int KI>
__device__ __forceinline__ void column_sum(const ItemHead<TG, KI>& h, const cplx<TG>* __restrict__ g, size_t zstride,
                                           int nbz, cplx<TG> (&acc)[KI]) {
#pragma unroll
    for (int it = 0; it < KI; ++it) acc[it] = mk((TG)0, (TG)0);
    if (h.uniform) {
        const cplx<TG>* gp = g + h.slab[0];
        for (int iz = 0; iz < nbz; ++iz) {
            const cplx<TG> v = gp[(size_t)iz * zstride];
#pragma unroll
            for (int it = 0; it < KI; ++it) fma_c(acc[it], h.ph[it][iz], v);
        }
    } else {
#pragma unroll
        for (int it = 0; it < KI; ++it)
            if (it < h.n_items)
                for (int iz = 0; iz < nbz; ++iz) fma_c(acc[it], h.ph[it][iz], g[h.slab[it] + (size_t)iz * zstride]);
    }
}

// W[i][blk][pair] for KI items x a tile of blockDim pairs, with the
// tight-binding epilogue in TG (psi_nm = conj(phi_n) phi_m from N phases per
// k-point, dt = C (tau_m - tau_n)):
//     H = psi X_0,  A_b = psi X_{4+b}                 (staged in shared memory)
//     H_a = i (psi X_{1+a} + dt_a H),  Om_q = i (psi X_{7+q} + dt_qa A_qb - dt_qb A_qa)
// Each thread reads back only its own staged values.  Only the upper triangle
// (n <= m) of each block is formed: every block is Hermitian and its consumers
// (the eigensolver, the rotation) read that triangle.  The FP32 H block is not
// written in the mixed form: its Jacobi reads the FP64 H(k).
template <typename T, typename TG, int NB, int KI>
__global__ void __launch_bounds__(128) sep_w_kernel(DevModel m, KRange kr, const cplx<TG>* __restrict__ G2, int nbz,
                                                    int rz0, int qx0, int nqx, cplx<T>* __restrict__ W) {
    extern __shared__ unsigned char smem_raw[];
    cplx<TG>* Xs = reinterpret_cast<cplx<TG>*>(smem_raw);  // [H, A_x, A_y, A_z][KI][blockDim]
    __shared__ ItemHead<TG, KI> h;
    const int NN = m.N * m.N, PT = blockDim.x, t = threadIdx.x;
    load_items<TG, KI>(h, kr, nbz, rz0, (size_t)nbz * NB * NN, m.has_tau ? m.tau : nullptr, m.N, qx0, nqx);
    // every block is Hermitian and its consumers read the upper triangle: the
    // CTA's threads take the elements n <= m of its pair tile (blockIdx.y)
    const int u = blockIdx.y * PT + t;
    if (u >= m.N * (m.N + 1) / 2) return;
    {
        int n, mm;
        upper_pair(u, m.N, n, mm);
        const int pair = n * m.N + mm;
        TG dt[3] = {(TG)0, (TG)0, (TG)0};
        cplx<TG> psi[KI];
#pragma unroll
        for (int it = 0; it < KI; ++it) psi[it] = mk((TG)1, (TG)0);
        if (m.has_tau) {
            double d[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) d[i] = m.tau[mm * 3 + i] - m.tau[n * 3 + i];
#pragma unroll
            for (int a = 0; a < 3; ++a) dt[a] = (TG)(m.C[a * 3 + 0] * d[0] + m.C[a * 3 + 1] * d[1] + m.C[a * 3 + 2] * d[2]);
#pragma unroll
            for (int it = 0; it < KI; ++it) psi[it] = cj_mul(h.phi[it][n], h.phi[it][mm]);
        }
        const int64_t i0 = (int64_t)blockIdx.x * KI;
        auto Wp = [&](int it, int b) { return W + ((size_t)(i0 + it) * NB + b) * NN + pair; };
        auto Xp = [&](int slot, int it) -> cplx<TG>& { return Xs[((size_t)slot * KI + it) * PT + t]; };
        cplx<TG> acc[KI];
        // H, then the connection A_b
        column_sum<TG, KI>(h, G2 + pair, (size_t)NB * NN, nbz, acc);
#pragma unroll
        for (int it = 0; it < KI; ++it) {
            const cplx<TG> v = psi[it] * acc[it];
            Xp(0, it) = v;
            if (sizeof(T) == 8 && it < h.n_items) *Wp(it, 0) = mk((T)v.re, (T)v.im);
        }
        if constexpr (NB == 10) {
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                column_sum<TG, KI>(h, G2 + (size_t)(4 + b) * NN + pair, (size_t)NB * NN, nbz, acc);
#pragma unroll
                for (int it = 0; it < KI; ++it) {
                    const cplx<TG> v = psi[it] * acc[it];
                    Xp(1 + b, it) = v;
                    if (it < h.n_items) *Wp(it, 4 + b) = mk((T)v.re, (T)v.im);
                }
            }
        }
        // H_a
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            column_sum<TG, KI>(h, G2 + (size_t)(1 + a) * NN + pair, (size_t)NB * NN, nbz, acc);
#pragma unroll
            for (int it = 0; it < KI; ++it) {
                const cplx<TG> v = times_i(psi[it] * acc[it] + dt[a] * Xp(0, it));
                if (it < h.n_items) *Wp(it, 1 + a) = mk((T)v.re, (T)v.im);
            }
        }
        // Omega_q, q = (x,y), (x,z), (y,z)
        if constexpr (NB == 10) {
            constexpr int qa[3] = {0, 0, 1}, qb[3] = {1, 2, 2};
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                column_sum<TG, KI>(h, G2 + (size_t)(7 + q) * NN + pair, (size_t)NB * NN, nbz, acc);
#pragma unroll
                for (int it = 0; it < KI; ++it) {
                    const cplx<TG> v = times_i(psi[it] * acc[it] + dt[qa[q]] * Xp(1 + qb[q], it) - dt[qb[q]] * Xp(1 + qa[q], it));
                    if (it < h.n_items) *Wp(it, 7 + q) = mk((T)v.re, (T)v.im);
                }
            }
        }
    }
}

// Hdf[i][pair] = psi * sum_iz phase(kz) G2d[qx][qy][iz][0][pair] for KI items,
// the FP64 H(k) of the mixed form, in double-FP32: the FP64 slab values and
// phases are split into FP32 hi + lo parts, each product a b of two such
// pairs is formed as p + e (p = ah bh, e = fma(ah, bh, -p) + ah bl + al bh),
// and the nbz-term sums run in TwoSum -- about 2^-44 relative, far below what
// the eigenpair refinement needs from H(k), with no FP64 arithmetic per term.
struct DFc {
    DF re, im;
};
__device__ __forceinline__ void split_d(double x, float& h, float& l) {
    h = __double2float_rn(x);
    l = __double2float_rn(x - (double)h);
}
// acc += (ah + al)(bh + bl)
__device__ __forceinline__ void df_mac(DF& acc, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    df_add(acc, p);
    acc.c = __fadd_rn(acc.c, e);
}
// acc += a b for complex a = (ar, ai) hi/lo and b likewise
__device__ __forceinline__ void dfc_mac(DFc& acc, const cplx<float>& ah, const cplx<float>& al, const cplx<float>& bh,
                                        const cplx<float>& bl) {
    df_mac(acc.re, ah.re, al.re, bh.re, bl.re);
    df_mac(acc.re, -ah.im, -al.im, bh.im, bl.im);
    df_mac(acc.im, ah.re, al.re, bh.im, bl.im);
    df_mac(acc.im, ah.im, al.im, bh.re, bl.re);
}
__device__ __forceinline__ void dfc_split(const DFc& v, cplx<float>& h, cplx<float>& l) {
    // renormalise each part so that hi carries the leading bits
    const float rh = __fadd_rn(v.re.s, v.re.c), ih = __fadd_rn(v.im.s, v.im.c);
    h = mk(rh, ih);
    l = mk(__fadd_rn(__fsub_rn(v.re.s, rh), v.re.c), __fadd_rn(__fsub_rn(v.im.s, ih), v.im.c));
}

template <int KI>
__global__ void __launch_bounds__(128) sep_h64_df_kernel(const cplx<double>* __restrict__ G2, KRange kr, int N,
                                                         int nbd, int nbz, int rz0, const double* __restrict__ tau,
                                                         int qx0, int nqx, float4* __restrict__ Hdf) {
    __shared__ ItemHead<double, KI> h;
    __shared__ cplx<float> phh[KI][32], phl[KI][32], fih[KI][kMaxN], fil[KI][kMaxN];
    const int NN = N * N;
    load_items<double, KI>(h, kr, nbz, rz0, (size_t)nbz * nbd * NN, tau, N, qx0, nqx);
    for (int e = threadIdx.x; e < KI * 32; e += blockDim.x) {
        const int it = e / 32, iz = e % 32;
        split_d(h.ph[it][iz].re, phh[it][iz].re, phl[it][iz].re);
        split_d(h.ph[it][iz].im, phh[it][iz].im, phl[it][iz].im);
    }
    if (tau)
        for (int e = threadIdx.x; e < KI * N; e += blockDim.x) {
            const int it = e / N, n = e % N;
            split_d(h.phi[it][n].re, fih[it][n].re, fil[it][n].re);
            split_d(h.phi[it][n].im, fih[it][n].im, fil[it][n].im);
        }
    __syncthreads();
    const size_t zs = (size_t)nbd * NN;
    const int NU = N * (N + 1) / 2;
    for (int u = threadIdx.x; u < NU; u += blockDim.x) {
        int n, mm;
        upper_pair(u, N, n, mm);
        const int pair = n * N + mm;
        DFc acc[KI];
#pragma unroll
        for (int it = 0; it < KI; ++it) acc[it] = DFc{DF{0.f, 0.f}, DF{0.f, 0.f}};
        if (h.uniform) {
            const cplx<double>* gp = G2 + pair + h.slab[0];
            for (int iz = 0; iz < nbz; ++iz) {
                const cplx<double> v = gp[(size_t)iz * zs];
                cplx<float> vh, vl;
                split_d(v.re, vh.re, vl.re);
                split_d(v.im, vh.im, vl.im);
#pragma unroll
                for (int it = 0; it < KI; ++it) dfc_mac(acc[it], phh[it][iz], phl[it][iz], vh, vl);
            }
        } else {
#pragma unroll
            for (int it = 0; it < KI; ++it)
                if (it < h.n_items)
                    for (int iz = 0; iz < nbz; ++iz) {
                        const cplx<double> v = G2[pair + h.slab[it] + (size_t)iz * zs];
                        cplx<float> vh, vl;
                        split_d(v.re, vh.re, vl.re);
                        split_d(v.im, vh.im, vl.im);
                        dfc_mac(acc[it], phh[it][iz], phl[it][iz], vh, vl);
                    }
        }
        const int64_t i0 = (int64_t)blockIdx.x * KI;
#pragma unroll
        for (int it = 0; it < KI; ++it) {
            if (it >= h.n_items) break;
            DFc r = acc[it];
            if (tau) {
                // psi = conj(phi_n) phi_m, then psi * X
                const cplx<float> an_h = conjg(fih[it][n]), an_l = conjg(fil[it][n]);
                DFc ps{DF{0.f, 0.f}, DF{0.f, 0.f}};
                dfc_mac(ps, an_h, an_l, fih[it][mm], fil[it][mm]);
                cplx<float> psh, psl, xh, xl;
                dfc_split(ps, psh, psl);
                dfc_split(r, xh, xl);
                r = DFc{DF{0.f, 0.f}, DF{0.f, 0.f}};
                dfc_mac(r, psh, psl, xh, xl);
            }
            cplx<float> xh, xl;
            dfc_split(r, xh, xl);
            Hdf[(size_t)(i0 + it) * NN + pair] = make_float4(xh.re, xh.im, xl.re, xl.im);
        }
    }
}

constexpr int kItemsF = 8;   // items per CTA with FP32 slabs
constexpr int kItemsD = 4;   // items per CTA with FP64 slabs
constexpr int kItemsH = 8;   // items per CTA of the FP64 H sums

}  // namespace

namespace {
// the integer R box of the model; false when R is not integer or the box is wider than 32
bool sep_box(const DevModel& m, const double* R_host, int lo[3], int nb[3]) {
    int hi[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    lo[0] = lo[1] = lo[2] = 1 << 30;
    for (int r = 0; r < m.nR; ++r)
        for (int a = 0; a < 3; ++a) {
            const double v = R_host[3 * r + a];
            if (std::fabs(v - std::rint(v)) > 1e-9 || std::fabs(v) > 1e6) return false;
            lo[a] = std::min(lo[a], (int)std::lrint(v));
            hi[a] = std::max(hi[a], (int)std::lrint(v));
        }
    for (int a = 0; a < 3; ++a) nb[a] = hi[a] - lo[a] + 1;
    return nb[0] <= 32 && nb[1] <= 32 && nb[2] <= 32;
}
}  // namespace

size_t sep_plan_want(const DevModel& m, const double* R_host, const int mp[3], bool fp64) {
    int lo[3], nb[3];
    if (!sep_box(m, R_host, lo, nb)) return 0;
    const size_t EL = (size_t)m.nb * m.N * m.N, NN = (size_t)m.N * m.N;
    const size_t box = (size_t)nb[0] * nb[1] * nb[2] * EL * sizeof(cplx<double>);
    const size_t g1 = (size_t)nb[1] * nb[2] * EL * sizeof(cplx<double>);
    const size_t g2f = fp64 ? 0 : (size_t)mp[1] * nb[2] * EL * sizeof(cplx<float>);
    const size_t g2d = (size_t)mp[1] * nb[2] * m.nb * NN * sizeof(cplx<double>);
    return box + (size_t)mp[0] * (g1 + g2f + g2d);
}

int sep_plan_build(SepPlan& p, const DevModel& m, const double* R_host, const cplx<double>* S_host, const int mp[3],
                   bool fp64, size_t budget, cudaStream_t s) {
    if (p.ready && p.fp64 == fp64 && p.mp[0] == mp[0] && p.mp[1] == mp[1] && p.mp[2] == mp[2]) return 0;
    sep_plan_free(p);
    int lo[3], nb[3];
    if (!sep_box(m, R_host, lo, nb)) return 1;
    const int NN = m.N * m.N, nbk = m.nb, EL = nbk * NN;
    const size_t box = (size_t)nb[0] * nb[1] * nb[2];
    const size_t box_bytes = box * EL * sizeof(cplx<double>);
    // bytes per qx of the slab arrays
    const size_t g1_q = (size_t)nb[1] * nb[2] * EL * sizeof(cplx<double>);
    const size_t g2f_q = fp64 ? 0 : (size_t)mp[1] * nb[2] * EL * sizeof(cplx<float>);
    auto g2d_q = [&](int nbd_) { return (size_t)mp[1] * nb[2] * nbd_ * NN * sizeof(cplx<double>); };
    if (budget == 0) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 2;
        budget = free_b / 2;   // the rest is left to the per-chunk buffers
    }
    if (box_bytes >= budget) return 1;
    const size_t room = budget - box_bytes;
    // The whole mesh in one slab when it fits -- for the mixed form with FP64
    // slabs of every block, so that its FP64 reruns take the separable sums
    // too -- else slabs of nqx consecutive qx, built one after the other
    // during the run (the mixed form then keeps FP64 slabs of H alone).
    int nbd = fp64 ? nbk : 1, nqx = 0;
    if (!fp64 && (size_t)mp[0] * (g1_q + g2f_q + g2d_q(nbk)) <= room) {
        nbd = nbk;
        nqx = mp[0];
    } else {
        const size_t per = g1_q + g2f_q + g2d_q(nbd);
        nqx = (int)std::min<size_t>((size_t)mp[0], room / per);
        if (nqx < 1) return 1;
    }
    std::vector<cplx<double>> hb(box * EL, mk(0.0, 0.0));
    for (int r = 0; r < m.nR; ++r) {
        const int ix = (int)std::lrint(R_host[3 * r]) - lo[0], iy = (int)std::lrint(R_host[3 * r + 1]) - lo[1],
                  iz = (int)std::lrint(R_host[3 * r + 2]) - lo[2];
        cplx<double>* cell = hb.data() + (((size_t)ix * nb[1] + iy) * nb[2] + iz) * EL;
        for (int pr = 0; pr < NN; ++pr)
            for (int b = 0; b < nbk; ++b) {
                cplx<double>& d = cell[(size_t)b * NN + pr];
                d = d + S_host[((size_t)r * NN + pr) * nbk + b];
            }
    }
    auto fail = [&](int rc) {
        sep_plan_free(p);
        return rc;
    };
    if (cudaMalloc(&p.box, box_bytes) != cudaSuccess) return fail(3);
    if (cudaMalloc(&p.G1, (size_t)nqx * g1_q) != cudaSuccess) return fail(3);
    if (cudaMalloc(&p.G2d, (size_t)nqx * g2d_q(nbd)) != cudaSuccess) return fail(3);
    if (!fp64 && cudaMalloc(&p.G2f, (size_t)nqx * g2f_q) != cudaSuccess) return fail(3);
    if (cudaMemcpyAsync(p.box, hb.data(), box_bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) return fail(2);
    for (int a = 0; a < 3; ++a) {
        p.mp[a] = mp[a];
        p.lo[a] = lo[a];
        p.nb[a] = nb[a];
    }
    p.N = m.N;
    p.nbk = nbk;
    p.nbd = nbd;
    p.nqx = nqx;
    p.fp64 = fp64;
    p.tau = m.has_tau ? m.tau : nullptr;
    p.h2d_bytes = box_bytes;
    p.dev_bytes = box_bytes + (size_t)nqx * (g1_q + g2f_q + g2d_q(nbd));
    p.built_qx0 = -1;
    if (nqx == mp[0] && launch_sep_slab(p, 0, s) != cudaSuccess) return fail(2);
    // the host box is read by the copy above: wait for it before it goes
    if (cudaStreamSynchronize(s) != cudaSuccess) return fail(2);
    p.ready = true;
    return 0;
}

// sep_stage_b for the mixed form's plans, in double-FP32: G1 arrives as hi/lo
// FP32 pairs (sep_stage_a with df_out), the ky phases are split once per CTA,
// and the nby-term sums run in TwoSum/TwoProduct FP32 arithmetic (about 2^-46
// relative) instead of on the 1/64-rate FP64 pipe.  G2f gets the FP32 rounding
// of the sum, G2d (the first nbd blocks) the pair widened to FP64.
__global__ void sep_stage_b_df(const float4* __restrict__ G1, cplx<double>* __restrict__ G2d,
                               cplx<float>* __restrict__ G2f, int NN, int nbk, int nbd, int nby, int nbz, int ry0,
                               int n1, int n2) {
    const int iz = blockIdx.y % nbz, qy = blockIdx.y / nbz, qx = blockIdx.z;
    __shared__ cplx<float> phh[32], phl[32];
    if (threadIdx.x < nby) {
        const cplx<double> p = phase(mp_coord(qy, n2), ry0 + (int)threadIdx.x);
        split_d(p.re, phh[threadIdx.x].re, phl[threadIdx.x].re);
        split_d(p.im, phh[threadIdx.x].im, phl[threadIdx.x].im);
    }
    __syncthreads();
    const int EL = nbk * NN;
    const size_t cell = ((size_t)qx * n2 + qy) * nbz + iz;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < EL; e += gridDim.x * blockDim.x) {
        DFc acc{DF{0.f, 0.f}, DF{0.f, 0.f}};
        for (int iy = 0; iy < nby; ++iy) {
            const float4 x = G1[(((size_t)qx * nby + iy) * nbz + iz) * EL + e];
            dfc_mac(acc, phh[iy], phl[iy], mk(x.x, x.y), mk(x.z, x.w));
        }
        cplx<float> h, l;
        dfc_split(acc, h, l);
        if (e < nbd * NN) G2d[cell * nbd * NN + e] = mk((double)h.re + (double)l.re, (double)h.im + (double)l.im);
        G2f[cell * EL + e] = h;
    }
}

cudaError_t launch_sep_slab(SepPlan& p, int qx0, cudaStream_t s) {
    const int nq = std::min(p.nqx, p.mp[0] - qx0);
    if (nq <= 0) return cudaErrorInvalidValue;
    const int EL = p.nbk * p.N * p.N;
    dim3 ga((EL + 255) / 256, p.nb[1] * p.nb[2], nq);
    // the mixed form's plans (FP32 slabs for the per-k work, FP64 slabs that feed
    // the double-FP32 H(k) and the FP64 reruns) are summed in double-FP32; the
    // FP64 form's plans in FP64
    const bool df = !p.fp64 && p.G2f;
    sep_stage_a<<<ga, 256, 0, s>>>(p.box, p.G1, EL, p.nb[0], p.nb[1], p.nb[2], p.lo[0], p.mp[0], qx0, df);
    dim3 gb((EL + 255) / 256, p.mp[1] * p.nb[2], nq);
    if (df)
        sep_stage_b_df<<<gb, 256, 0, s>>>(reinterpret_cast<const float4*>(p.G1), p.G2d, p.G2f, p.N * p.N, p.nbk, p.nbd,
                                          p.nb[1], p.nb[2], p.lo[1], p.mp[0], p.mp[1]);
    else
        sep_stage_b<<<gb, 256, 0, s>>>(p.G1, p.G2d, p.G2f, p.N * p.N, p.nbk, p.nbd, p.nb[1], p.nb[2], p.lo[1], p.mp[0],
                                       p.mp[1]);
    p.built_qx0 = qx0;
    return cudaGetLastError();
}

void sep_plan_free(SepPlan& p) {
    for (void* q : {(void*)p.G2d, (void*)p.G2f, (void*)p.G1, (void*)p.box})
        if (q) cudaFree(q);
    p = SepPlan();
}

namespace {
inline int pair_tile(int n_elem) { return n_elem >= 128 ? 128 : ((n_elem + 31) / 32) * 32; }

template <typename T, typename TG, int NB, int KI>
cudaError_t launch_w(const DevModel& m, const KRange& kr, const cplx<TG>* G2, int nbz, int rz0, int qx0, int nqx,
                     cplx<T>* W, cudaStream_t s) {
    const int NU = m.N * (m.N + 1) / 2, PT = pair_tile(NU);
    const size_t smem = (size_t)(NB == 10 ? 4 : 1) * KI * PT * sizeof(cplx<TG>);
    cudaError_t e = cudaFuncSetAttribute(sep_w_kernel<T, TG, NB, KI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    // one pair tile per CTA: the kernel streams its W-gauge output, and the
    // measured time is lowest with the most CTAs in flight
    dim3 grid((unsigned)((kr.count + KI - 1) / KI), (unsigned)((NU + PT - 1) / PT));
    sep_w_kernel<T, TG, NB, KI><<<grid, PT, smem, s>>>(m, kr, G2, nbz, rz0, qx0, nqx, W);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_sep_h64(const SepPlan& p, const KRange& kr, float4* Hdf, cudaStream_t s) {
    if (kr.count <= 0) return cudaSuccess;
    const int NU = p.N * (p.N + 1) / 2, PT = pair_tile(NU);
    sep_h64_df_kernel<kItemsH><<<(unsigned)((kr.count + kItemsH - 1) / kItemsH), PT, 0, s>>>(
        p.G2d, kr, p.N, p.nbd, p.nb[2], p.lo[2], p.tau, p.built_qx0, p.nqx, Hdf);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_sep_w(const SepPlan& p, const DevModel& m, const KRange& kr, cplx<T>* W, cudaStream_t s) {
    if (kr.count <= 0) return cudaSuccess;
    if (sizeof(T) == 8) {
        if (p.nbd != p.nbk) return cudaErrorInvalidValue;  // FP64 output needs FP64 slabs of every block
        if (m.nb == 10) return launch_w<T, double, 10, kItemsD>(m, kr, p.G2d, p.nb[2], p.lo[2], p.built_qx0, p.nqx, W, s);
        return launch_w<T, double, 4, kItemsD>(m, kr, p.G2d, p.nb[2], p.lo[2], p.built_qx0, p.nqx, W, s);
    }
    if (m.nb == 10) return launch_w<T, float, 10, kItemsF>(m, kr, p.G2f, p.nb[2], p.lo[2], p.built_qx0, p.nqx, W, s);
    return launch_w<T, float, 4, kItemsF>(m, kr, p.G2f, p.nb[2], p.lo[2], p.built_qx0, p.nqx, W, s);
}

template cudaError_t launch_sep_w<double>(const SepPlan&, const DevModel&, const KRange&, cplx<double>*, cudaStream_t);
template cudaError_t launch_sep_w<float>(const SepPlan&, const DevModel&, const KRange&, cplx<float>*, cudaStream_t);

}  // namespace mepi
