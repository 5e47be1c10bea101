// W -> Hbar gauge rotation of rotate_gauge (src/wann_interp.f90:502-550):
//     Hbar_a = U^dag H_a U,   Abar_a = U^dag A_a U   (a = x,y,z; D1 position:
//     the connection is rotated from A_a itself, not from the stale buffer the
//     reference reuses at :531-533),
// and only the band diagonal of U^dag Omega_q U for the three independent
// curvature components -- the band sums consume no other part of Omega
// (src/mep_niu.f90:35, src/kubo_mep.f90:35), so the 54 zgemm per k of
// curv_gaugeTrafo collapse to 3 diagonal-only rotations here plus O(N^2)
// commutator diagonals in the gauge kernel.
//
// One k-point per CTA: U and the operand (mirrored from its upper triangle,
// every W-gauge block being Hermitian) are staged in shared memory (padded
// to an even size with zeros) and each product is an N x N x N complex
// contraction in which every thread computes 4 x 1 output tiles
// (smem_cgemm: broadcast loads of A, conflict-free loads of B, each feeding
// four multiply-adds).
// Without the gauge transformation the kernel copies the W-gauge blocks.
#include "mepi_internal.cuh"

namespace mepi {

namespace {

// A Hermitian W-gauge block into shared memory from its upper triangle (the
// lower one is not formed by the separable Fourier sums).
template <typename T>
__device__ __forceinline__ void load_hermitian(const cplx<T>* __restrict__ Wb, cplx<T>* Xs, int N, int ld, int tid,
                                               int nt) {
    const FastDiv byN(N);
    for (int e = tid; e < N * N; e += nt) {
        const int i = byN.div(e), c = e - i * N;
        if (i > c) continue;
        const cplx<T> x = Wb[e];
        Xs[i * ld + c] = x;
        if (i != c) Xs[c * ld + i] = conjg(x);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) rot_kernel(DevModel m, const cplx<T>* __restrict__ W,
                                                  const cplx<T>* __restrict__ Ug, cplx<T>* __restrict__ HA,
                                                  cplx<T>* __restrict__ OD) {
    extern __shared__ unsigned char smem_raw[];
    constexpr bool f32 = sizeof(T) == 4;
    const int N = m.N, NN = N * N;
    const int Np = N + (N & 1), ld = Np + 1;   // even padded size (zero padding), odd row stride
    cplx<T>* Us = reinterpret_cast<cplx<T>*>(smem_raw);
    cplx<T>* Xs = Us + Np * ld;
    cplx<T>* Ts = Xs + Np * ld;
    cplx<T>* Tl = Ts + Np * ld;   // FP32 form: low-order part of H_a U
    const int tid = threadIdx.x, nt = blockDim.x;
    const int64_t k = blockIdx.x;
    const int nbW = m.nb;
    const cplx<T>* Wk = W + (size_t)k * nbW * NN;
    const int nmat = m.has_r ? 6 : 3;
    cplx<T>* HAk = HA + (size_t)k * 6 * NN;
    const FastDiv byN(N);

    if (!m.do_gauge) {
        for (int j = 0; j < nmat; ++j)
            for (int e = tid; e < NN; e += nt) {
                const int i = e / N, c = e % N;
                if (i > c) continue;
                const cplx<T> x = Wk[(size_t)(1 + j) * NN + e];
                HAk[(size_t)j * NN + e] = x;
                if (i != c) HAk[(size_t)j * NN + c * N + i] = conjg(x);
            }
        if (m.has_r)
            for (int q = 0; q < 3; ++q)
                for (int n = tid; n < N; n += nt) OD[((size_t)k * 3 + q) * N + n] = Wk[(size_t)(7 + q) * NN + n * N + n];
        return;
    }
    const cplx<T> zero = mk((T)0, (T)0);
    for (int e = tid; e < Np * ld; e += nt) {
        const int i = e / ld, j = e % ld;
        Us[e] = (i < N && j < N) ? Ug[(size_t)k * NN + i * N + j] : zero;
        Xs[e] = zero;
        Ts[e] = zero;
        if (f32) Tl[e] = zero;
    }
    // blocks 1..3 (H_a) and 4..6 (A_a): full rotation
    for (int j = 0; j < nmat; ++j) {
        __syncthreads();
        load_hermitian(Wk + (size_t)(1 + j) * NN, Xs, N, ld, tid, nt);
        __syncthreads();
        if constexpr (f32) {
            if (j < 3) {
                // the velocity blocks in Dot2: T = X U (hi + lo), then the
                // Hermitian Y = U^dag T (upper triangle, mirrored)
                cgemm_dot2<false>(Np, ld, Xs, Us, nullptr, Ts, Tl, false, tid, nt);
                __syncthreads();
                cgemm_dot2<true>(Np, ld, Us, Ts, Tl, Xs, nullptr, true, tid, nt);
                __syncthreads();
                for (int e = tid; e < NN; e += nt) HAk[(size_t)j * NN + e] = Xs[byN.div(e) * ld + byN.mod(e)];
                continue;
            }
        }
        smem_cgemm<T, false>(Np, ld, Xs, Us, Ts, tid, nt);          // T = X U
        __syncthreads();
        smem_cgemm_herm<T>(Np, ld, Us, Ts, Xs, tid, nt);            // Y = U^dag T (Hermitian, into Xs)
        __syncthreads();
        for (int e = tid; e < NN; e += nt) HAk[(size_t)j * NN + e] = Xs[byN.div(e) * ld + byN.mod(e)];
    }
    if (!m.has_r) return;
    // blocks 7..9 (Omega_q): diagonal of U^dag Omega_q U only
    for (int q = 0; q < 3; ++q) {
        __syncthreads();
        load_hermitian(Wk + (size_t)(7 + q) * NN, Xs, N, ld, tid, nt);
        __syncthreads();
        smem_cgemm<T, false>(Np, ld, Xs, Us, Ts, tid, nt);          // T = Omega U
        __syncthreads();
        for (int n = tid; n < N; n += nt) {
            cplx<T> acc = zero;
            for (int l = 0; l < N; ++l) fma_cjc(acc, Us[l * ld + n], Ts[l * ld + n]);
            OD[((size_t)k * 3 + q) * N + n] = acc;
        }
    }
}

}  // namespace

template <typename T>
cudaError_t launch_rot(const DevModel& m, int64_t nk, const cplx<T>* W, const cplx<T>* U, cplx<T>* HA, cplx<T>* OD,
                       cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    const int Np = m.N + (m.N & 1);
    size_t smem = (sizeof(T) == 4 ? 4 : 3) * (size_t)Np * (Np + 1) * sizeof(cplx<T>);
    cudaError_t e = cudaFuncSetAttribute(rot_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(rot_kernel<T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    int threads = m.N <= 16 ? 128 : 256;
    rot_kernel<T><<<(unsigned)nk, threads, smem, s>>>(m, W, U, HA, OD);
    return cudaGetLastError();
}

template cudaError_t launch_rot<double>(const DevModel&, int64_t, const cplx<double>*, const cplx<double>*,
                                        cplx<double>*, cplx<double>*, cudaStream_t);
template cudaError_t launch_rot<float>(const DevModel&, int64_t, const cplx<float>*, const cplx<float>*, cplx<float>*,
                                       cplx<float>*, cudaStream_t);

}  // namespace mepi
