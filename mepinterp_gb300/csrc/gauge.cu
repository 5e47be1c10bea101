// Hbar -> H gauge step and velocity, per k-point:
//   get_gauge_covar_deriv (src/wann_interp.f90:565-617)
//       D_a(n,m) = Hbar_a(n,m) / (E_m - E_n)  if |E_m - E_n| > kuboTol, else 0
//   conn_gaugeTrafo (:620-633)   A^H_a = Abar_a + i D_a
//   curv_gaugeTrafo (:636-658), band diagonal only:
//       Om^H_ab(n,n) = Obar_ab(n,n) - [D_a, A'_b]_nn + [D_b, A'_a]_nn - i [D_a, D_b]_nn
//       with A' = A^H (semantics "ref", the reference's ordering, D4) or Abar ("paper")
//   get_velo (:406-444)
//       V_a(p,q) = Hbar_a(p,q) - i (E_q - E_p) A''_a(p,q)   (p != q)
//       A'' = A^H ("ref", D5) or Abar ("paper");  V_a(p,p) = Hbar_a(p,p) (D2);
//       without r(R): V = Hbar.
// plus the Chern-Simons per-band value of mep_niu_CS / kubo_mep_CS
// (src/mep_niu.f90:34-38, src/kubo_mep.f90:34-39):
//       csv(n) = 0.5 Re( sum_c conj(A^H_c(n,n)) om_c(n) ),
//       om = (2 Om_yz, -2 Om_xz, 2 Om_xy)  (= sum_ab eps_abc Om_ab, Om antisymmetric).
// Without the gauge transformation D = 0 and the W-gauge blocks are used.
#include "mepi_internal.cuh"

namespace mepi {

namespace {

// The six rotated blocks of one k-point (Hbar_x,y,z, Abar_x,y,z): staged in
// shared memory as real and imaginary planes with row stride N + 1, so that
// both row and column walks are free of bank conflicts, or, when they do not
// fit (FP64 beyond N = 46), read from global memory.
template <typename T>
struct GaugeSm {
    T* re;
    T* im;
    const cplx<T>* glob;
    const T* invd;   // [N][ld] 1/(E_m - E_n) where D is defined, else 0
    int N, ld, semantics;
    bool staged;
    __device__ __forceinline__ cplx<T> X(int blk, int n, int m) const {
        if (!staged) return glob[((size_t)blk * N + n) * N + m];
        const int o = (blk * N + n) * ld + m;
        return mk(re[o], im[o]);
    }
    __device__ __forceinline__ cplx<T> D(int a, int n, int m) const {
        const T w = invd[n * ld + m];
        const cplx<T> h = X(a, n, m);
        return mk(h.re * w, h.im * w);
    }
    // A' used in the curvature commutators, given D(a, n, m)
    __device__ __forceinline__ cplx<T> Ac(int a, int n, int m, const cplx<T>& d) const {
        const cplx<T> ab = X(3 + a, n, m);
        if (semantics != 0) return ab;
        return ab + times_i(d);
    }
};

template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__global__ void __launch_bounds__(256) gauge_kernel(DevModel m, const double* __restrict__ Eg, const cplx<T>* __restrict__ HA,
                                                    const cplx<T>* __restrict__ OD, cplx<T>* __restrict__ V,
                                                    T* __restrict__ CSV, cplx<T>* __restrict__ ODH, bool staged) {
    const int N = m.N, NN = N * N, ld = N + 1;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int64_t k = blockIdx.x;
    __shared__ double Es[kMaxN];
    __shared__ cplx<T> Oh[3][kMaxN];
    extern __shared__ unsigned char smem_raw[];
    T* invd = reinterpret_cast<T*>(smem_raw);
    T* Eh = invd + N * ld;   // energies as FP32 hi + lo (the FP32 form's velocity)
    T* El = Eh + N;
    GaugeSm<T> g;
    g.re = El + N;           // the staged planes (when they fit)
    g.im = g.re + 6 * N * ld;
    g.invd = invd;
    g.N = N;
    g.ld = ld;
    g.semantics = m.semantics;
    g.staged = staged;
    const int nblk = m.has_r ? 6 : 3;
    const cplx<T>* HAk = HA + (size_t)k * 6 * NN;
    g.glob = HAk;
    const FastDiv byN(N), byNN(NN);
    for (int n = tid; n < N; n += nt) {
        const double e = Eg[(size_t)k * N + n];
        Es[n] = e;
        Eh[n] = (T)e;
        El[n] = (T)(e - (double)(T)e);
    }
    if (staged) {
        // four loads in flight per thread before the shared-memory stores
        const int tot = nblk * NN;
        for (int e0 = tid; e0 < tot; e0 += 4 * nt) {
            cplx<T> x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int e = e0 + u * nt;
                x[u] = e < tot ? HAk[e] : mk((T)0, (T)0);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int e = e0 + u * nt;
                if (e >= tot) break;
                const int row = byN.div(e), col = e - row * N;   // row = blk * N + n
                const int o = row * ld + col;
                g.re[o] = x[u].re;
                g.im[o] = x[u].im;
            }
        }
    }
    __syncthreads();
    // inverse gaps of the covariant derivative: the kuboTol decision in FP64
    for (int e = tid; e < NN; e += nt) {
        const int n = byN.div(e), mm = e - n * N;
        const double ded = Es[mm] - Es[n];
        invd[n * ld + mm] = (m.do_gauge && n != mm && fabs(ded) > m.kubo_tol) ? (T)1 / (T)ded : (T)0;
    }
    __syncthreads();
    cplx<T>* Vk = V + (size_t)k * 3 * NN;
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    // the curvature diagonal (warps 0..2, one component q each, a lane per band
    // n summing over m: no cross-lane reduction, and both the row walk n -> (n, m)
    // and the column walk (m, n) are conflict-free in the padded planes) runs
    // beside the velocity (the other warps; all warps when there is no r(R))
    const bool curv = m.has_r && nw > 3;
    if (curv && warp < 3) {
        const int q = warp;
        const int a = q < 2 ? 0 : 1, b = q == 0 ? 1 : 2;   // (x,y), (x,z), (y,z)
        for (int n = lane; n < N; n += 32) {
            cplx<T> o = OD[((size_t)k * 3 + q) * N + n];
            if (m.do_gauge) {
                cplx<T> c1 = mk((T)0, (T)0), c2 = c1, c3 = c1;
                for (int mm = 0; mm < N; ++mm) {
                    if (mm == n) continue;  // D has no diagonal, so the m = n terms vanish
                    const cplx<T> Da_nm = g.D(a, n, mm), Da_mn = g.D(a, mm, n);
                    const cplx<T> Db_nm = g.D(b, n, mm), Db_mn = g.D(b, mm, n);
                    // [D_a, A'_b]_nn
                    fma_c(c1, Da_nm, g.Ac(b, mm, n, Db_mn));
                    c1 = c1 - g.Ac(b, n, mm, Db_nm) * Da_mn;
                    // [D_b, A'_a]_nn
                    fma_c(c2, Db_nm, g.Ac(a, mm, n, Da_mn));
                    c2 = c2 - g.Ac(a, n, mm, Da_nm) * Db_mn;
                    // [D_a, D_b]_nn
                    fma_c(c3, Da_nm, Db_mn);
                    c3 = c3 - Db_nm * Da_mn;
                }
                o = o - c1 + c2 - times_i(c3);
            }
            Oh[q][n] = o;
            if (ODH) ODH[((size_t)k * 3 + q) * N + n] = o;
        }
    } else {
        // velocity
        const int t0 = curv ? tid - 96 : tid, nv = curv ? nt - 96 : nt;
        for (int e = t0; e < 3 * NN; e += nv) {
            const int row = byN.div(e), a = byNN.div(e), p = row - a * N, q = e - row * N;
            const cplx<T> hb = g.X(a, p, q);
            cplx<T> v = hb;
            if (m.has_r && p != q) {
                const cplx<T> ab = g.X(3 + a, p, q);
                cplx<T> av = ab;
                if (m.semantics == 0 || !m.do_gauge) av = ab + times_i(g.D(a, p, q));
                T de;
                if constexpr (sizeof(T) == 8)
                    de = (T)(Es[q] - Es[p]);
                else   // E_q - E_p from the hi + lo pairs: exact for close energies
                    de = (Eh[q] - Eh[p]) + (El[q] - El[p]);
                v = hb - times_i(de * av);
            }
            Vk[e] = v;
        }
    }
    if (!m.has_r) {
        for (int n = tid; n < N; n += nt) CSV[(size_t)k * N + n] = (T)0;
        return;
    }
    if (!curv) {
        // fewer than four warps: the curvature diagonal after the velocity, one
        // warp per (q, n), lanes over m
        for (int t = warp; t < 3 * N; t += nw) {
            const int q = byN.div(t), n = t - q * N;
            const int a = q < 2 ? 0 : 1, b = q == 0 ? 1 : 2;
            cplx<T> o = OD[((size_t)k * 3 + q) * N + n];
            if (m.do_gauge) {
                cplx<T> c1 = mk((T)0, (T)0), c2 = c1, c3 = c1;
                for (int mm = lane; mm < N; mm += 32) {
                    if (mm == n) continue;
                    const cplx<T> Da_nm = g.D(a, n, mm), Da_mn = g.D(a, mm, n);
                    const cplx<T> Db_nm = g.D(b, n, mm), Db_mn = g.D(b, mm, n);
                    fma_c(c1, Da_nm, g.Ac(b, mm, n, Db_mn));
                    c1 = c1 - g.Ac(b, n, mm, Db_nm) * Da_mn;
                    fma_c(c2, Db_nm, g.Ac(a, mm, n, Da_mn));
                    c2 = c2 - g.Ac(a, n, mm, Da_nm) * Db_mn;
                    fma_c(c3, Da_nm, Db_mn);
                    c3 = c3 - Db_nm * Da_mn;
                }
                c1 = mk(warp_sum_t(c1.re), warp_sum_t(c1.im));
                c2 = mk(warp_sum_t(c2.re), warp_sum_t(c2.im));
                c3 = mk(warp_sum_t(c3.re), warp_sum_t(c3.im));
                o = o - c1 + c2 - times_i(c3);
            }
            if (lane == 0) {
                Oh[q][n] = o;
                if (ODH) ODH[((size_t)k * 3 + q) * N + n] = o;
            }
        }
    }
    __syncthreads();
    for (int n = tid; n < N; n += nt) {
        const cplx<T> om[3] = {(T)2 * Oh[2][n], (T)-2 * Oh[1][n], (T)2 * Oh[0][n]};
        cplx<T> acc = mk((T)0, (T)0);
        for (int c = 0; c < 3; ++c) fma_cjc(acc, g.X(3 + c, n, n), om[c]);
        CSV[(size_t)k * N + n] = (T)0.5 * acc.re;
    }
}

}  // namespace

template <typename T>
cudaError_t launch_gauge(const DevModel& m, int64_t nk, const double* E, const cplx<T>* HA, const cplx<T>* OD,
                         cplx<T>* V, T* CSV, cplx<T>* ODH, cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    int threads = m.N <= 16 ? 128 : 256;
    const size_t base = ((size_t)m.N * (m.N + 1) + 2 * (size_t)m.N) * sizeof(T);   // inverse gaps, energy pairs
    size_t smem = base + 2 * 6 * (size_t)m.N * (m.N + 1) * sizeof(T);
    const bool staged = smem <= (size_t)220 * 1024;   // the opt-in limit is 227 KB, static arrays included
    if (!staged) smem = base;
    cudaError_t e = cudaFuncSetAttribute(gauge_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    gauge_kernel<T><<<(unsigned)nk, threads, smem, s>>>(m, E, HA, OD, V, CSV, ODH, staged);
    return cudaGetLastError();
}

template cudaError_t launch_gauge<double>(const DevModel&, int64_t, const double*, const cplx<double>*,
                                          const cplx<double>*, cplx<double>*, double*, cplx<double>*, cudaStream_t);
template cudaError_t launch_gauge<float>(const DevModel&, int64_t, const double*, const cplx<float>*,
                                         const cplx<float>*, cplx<float>*, float*, cplx<float>*, cudaStream_t);

}  // namespace mepi
