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

template <typename T>
struct GaugeCtx {
    const cplx<T>* HA;  // [6][N][N] of this k
    const T* invd;      // [N][N] 1/(E_m - E_n) where D is defined, else 0 (shared memory)
    int N, semantics;
    __device__ __forceinline__ cplx<T> D(int a, int n, int m) const {
        const T w = invd[n * N + m];
        const cplx<T> h = HA[(size_t)a * N * N + n * N + m];
        return mk(h.re * w, h.im * w);
    }
    // A' used in the curvature commutators
    __device__ __forceinline__ cplx<T> Ac(int a, int n, int m) const {
        cplx<T> ab = HA[(size_t)(3 + a) * N * N + n * N + m];
        if (semantics != 0) return ab;
        return ab + times_i(D(a, n, m));
    }
};

template <typename T>
__global__ void __launch_bounds__(256) gauge_kernel(DevModel m, const double* __restrict__ Eg, const cplx<T>* __restrict__ HA,
                                                    const cplx<T>* __restrict__ OD, cplx<T>* __restrict__ V,
                                                    T* __restrict__ CSV, cplx<T>* __restrict__ ODH) {
    const int N = m.N, NN = N * N;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int64_t k = blockIdx.x;
    __shared__ double Es[kMaxN];
    __shared__ cplx<T> Oh[3][kMaxN];
    extern __shared__ unsigned char smem_raw[];
    T* invd = reinterpret_cast<T*>(smem_raw);
    for (int n = tid; n < N; n += nt) Es[n] = Eg[(size_t)k * N + n];
    __syncthreads();
    // inverse gaps of the covariant derivative, decided and formed in FP64
    for (int e = tid; e < NN; e += nt) {
        const int n = e / N, mm = e % N;
        const double ded = Es[mm] - Es[n];
        invd[e] = (m.do_gauge && n != mm && fabs(ded) > m.kubo_tol) ? (T)(1.0 / ded) : (T)0;
    }
    __syncthreads();
    GaugeCtx<T> g;
    g.HA = HA + (size_t)k * 6 * NN;
    g.invd = invd;
    g.N = N;
    g.semantics = m.semantics;
    cplx<T>* Vk = V + (size_t)k * 3 * NN;
    // velocity
    for (int e = tid; e < 3 * NN; e += nt) {
        int a = e / NN, p = (e / N) % N, q = e % N;
        cplx<T> hb = g.HA[e];
        cplx<T> v = hb;
        if (m.has_r && p != q) {
            cplx<T> ab = g.HA[(size_t)(3 + a) * NN + p * N + q];
            cplx<T> av = ab;
            if (m.semantics == 0 || !m.do_gauge) av = ab + times_i(g.D(a, p, q));
            const T de = (T)(Es[q] - Es[p]);
            v = hb - times_i(de * av);
        }
        Vk[e] = v;
    }
    if (!m.has_r) {
        for (int n = tid; n < N; n += nt) CSV[(size_t)k * N + n] = (T)0;
        return;
    }
    // curvature diagonal
    const int qa[3] = {0, 0, 1}, qb[3] = {1, 2, 2};
    for (int t = tid; t < 3 * N; t += nt) {
        int q = t / N, n = t % N;
        int a = qa[q], b = qb[q];
        cplx<T> o = OD[((size_t)k * 3 + q) * N + n];
        if (m.do_gauge) {
            cplx<T> c1 = mk((T)0, (T)0), c2 = c1, c3 = c1;
            for (int mm = 0; mm < N; ++mm) {
                if (mm == n) continue;  // D has no diagonal, so the m = n terms vanish
                cplx<T> Da_nm = g.D(a, n, mm), Da_mn = g.D(a, mm, n);
                cplx<T> Db_nm = g.D(b, n, mm), Db_mn = g.D(b, mm, n);
                // [D_a, A'_b]_nn
                fma_c(c1, Da_nm, g.Ac(b, mm, n));
                c1 = c1 - g.Ac(b, n, mm) * Da_mn;
                // [D_b, A'_a]_nn
                fma_c(c2, Db_nm, g.Ac(a, mm, n));
                c2 = c2 - g.Ac(a, n, mm) * Db_mn;
                // [D_a, D_b]_nn
                fma_c(c3, Da_nm, Db_mn);
                c3 = c3 - Db_nm * Da_mn;
            }
            o = o - c1 + c2 - times_i(c3);
        }
        Oh[q][n] = o;
        if (ODH) ODH[((size_t)k * 3 + q) * N + n] = o;
    }
    __syncthreads();
    for (int n = tid; n < N; n += nt) {
        cplx<T> om[3] = {(T)2 * Oh[2][n], (T)-2 * Oh[1][n], (T)2 * Oh[0][n]};
        cplx<T> acc = mk((T)0, (T)0);
        for (int c = 0; c < 3; ++c) fma_cjc(acc, g.HA[(size_t)(3 + c) * NN + n * N + n], om[c]);
        CSV[(size_t)k * N + n] = (T)0.5 * acc.re;
    }
}

}  // namespace

template <typename T>
cudaError_t launch_gauge(const DevModel& m, int64_t nk, const double* E, const cplx<T>* HA, const cplx<T>* OD,
                         cplx<T>* V, T* CSV, cplx<T>* ODH, cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    int threads = m.N <= 16 ? 128 : 256;
    const size_t smem = (size_t)m.N * m.N * sizeof(T);
    cudaError_t e = cudaFuncSetAttribute(gauge_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    gauge_kernel<T><<<(unsigned)nk, threads, smem, s>>>(m, E, HA, OD, V, CSV, ODH);
    return cudaGetLastError();
}

template cudaError_t launch_gauge<double>(const DevModel&, int64_t, const double*, const cplx<double>*,
                                          const cplx<double>*, cplx<double>*, double*, cplx<double>*, cudaStream_t);
template cudaError_t launch_gauge<float>(const DevModel&, int64_t, const double*, const cplx<float>*,
                                         const cplx<float>*, cplx<float>*, float*, cplx<float>*, cudaStream_t);

}  // namespace mepi
