// Batched Hermitian eigensolver replacing zheevd_wrapper
// (src/matrix_math.f90:192-226: jobz='V', uplo='U', eigenvalues ascending,
// eigenvectors in the columns of U).
//
// One k-point per CTA.  The matrix and the eigenvector accumulator live in
// shared memory; each sweep of the two-sided cyclic Jacobi method runs as N-1
// rounds of N/2 disjoint plane rotations (round-robin "circle" ordering), all
// pairs of a round rotated at once (a numpy emulation of exactly this scheme
// converges in 5-8 FP64 / 4-7 FP32 sweeps at N = 8..64).  For a pair (p,q) with M_pq = g e^{i phi}
// the rotation is G = [[c, s e^{i phi}], [-s e^{-i phi}, c]] with the
// Rutishauser choice t = sgn(theta)/(|theta| + sqrt(1+theta^2)),
// theta = (M_qq - M_pp)/(2g), c = 1/sqrt(1+t^2), s = t c; M <- G^dag M G and
// U <- U G.  The input is Hermitised from the upper triangle as LAPACK's 'U'
// option reads it.  Sweeps stop once the off-diagonal Frobenius norm falls
// below 4 sqrt(N) eps ||H||_F, or at max_sweeps: hitting the cap raises flag_cap (the
// caller turns it into MEPI_ERR_EIG or, in the mixed form, an FP64 rerun of
// that k-point); every loop is bounded.
#include "mepi_internal.cuh"

namespace mepi {

namespace {

// Stop when ||offdiag(M)||_F <= 4 sqrt(N) eps ||H||_F (the rounding floor of the
// off-diagonal entries); rotations with |M_pq| below skip * ||H||_F are skipped
// (their phase e^{i phi} would not be unitary to working precision).
template <typename T> struct EigTol;
template <> struct EigTol<double> { static constexpr double eps = 2.220446049250313e-16, skip = 1e-20; };
template <> struct EigTol<float> { static constexpr double eps = 1.1920928955078125e-07, skip = 1e-10; };

template <typename T>
__global__ void __launch_bounds__(256) jacobi_kernel(int N, const cplx<T>* __restrict__ W, int nbW,
                                                     T* __restrict__ E, cplx<T>* __restrict__ U, int max_sweeps,
                                                     int* sweeps_max, int* flag_cap, double degen_gap,
                                                     int* redo_flag) {
    extern __shared__ unsigned char smem_raw[];
    const int ld = N + 1;                       // padded row stride
    cplx<T>* M = reinterpret_cast<cplx<T>*>(smem_raw);
    cplx<T>* Vv = M + N * ld;
    T* cs = reinterpret_cast<T*>(Vv + N * ld);  // per pair: c, s
    T* ss = cs + kMaxN / 2;
    cplx<T>* eph = reinterpret_cast<cplx<T>*>(ss + kMaxN / 2);  // e^{i phi}
    T* dnew = reinterpret_cast<T*>(eph + kMaxN / 2);           // new diagonal (2 per pair)
    int* pp = reinterpret_cast<int*>(dnew + kMaxN);
    int* qq = pp + kMaxN / 2;
    T* red = reinterpret_cast<T*>(qq + kMaxN / 2);            // reduction scratch [256]
    __shared__ int s_conv;

    const int tid = threadIdx.x, nt = blockDim.x;
    const int64_t k = blockIdx.x;
    const cplx<T>* Hk = W + (size_t)k * nbW * N * N;
    const int NN = N * N;
    // load, Hermitise from the upper triangle
    for (int e = tid; e < NN; e += nt) {
        int i = e / N, j = e % N;
        cplx<T> v;
        if (i < j) v = Hk[i * N + j];
        else if (i > j) v = conjg(Hk[j * N + i]);
        else v = mk(Hk[i * N + i].re, (T)0);
        M[i * ld + j] = v;
        Vv[i * ld + j] = mk((T)(i == j ? 1 : 0), (T)0);
    }
    // ||H||_F^2
    T part = 0;
    for (int e = tid; e < NN; e += nt) {
        int i = e / N, j = e % N;
        part += abs2(M[i * ld + j]);
    }
    red[tid] = part;
    __syncthreads();
    for (int w = nt / 2; w > 0; w >>= 1) {
        if (tid < w) red[tid] += red[tid + w];
        __syncthreads();
    }
    const T fro2 = red[0];
    __syncthreads();

    const int Np = N + (N & 1);
    const int half = Np / 2;
    const int Np1 = Np - 1;
    const T tolr = (T)(4.0 * EigTol<T>::eps) * sqrt((T)N);
    const T tol2 = tolr * tolr * fro2;
    const T gskip = (T)EigTol<T>::skip * sqrt(fro2);
    int sweep = 0;
    bool converged = (N == 1);
    for (sweep = 0; sweep < max_sweeps && !converged; ++sweep) {
        for (int r = 0; r < Np1; ++r) {
            // 1. rotation parameters for the pairs of this round
            if (tid < half) {
                int a, b;
                if (tid == 0) { a = Np1; b = r; }
                else { a = (r + tid) % Np1; b = (r - tid + Np1) % Np1; }
                int p = a < b ? a : b, q = a < b ? b : a;
                T c = 1, s = 0;
                cplx<T> ph = mk((T)1, (T)0);
                if (q < N) {
                    T app = M[p * ld + p].re, aqq = M[q * ld + q].re;
                    cplx<T> apq = M[p * ld + q];
                    T g = sqrt(abs2(apq));
                    if (g > gskip) {
                        T theta = (aqq - app) / (2 * g);
                        T t = (theta >= 0 ? (T)1 : (T)-1) / (fabs(theta) + sqrt((T)1 + theta * theta));
                        c = (T)1 / sqrt((T)1 + t * t);
                        s = t * c;
                        ph = mk(apq.re / g, apq.im / g);
                        dnew[2 * tid] = app - t * g;
                        dnew[2 * tid + 1] = aqq + t * g;
                    } else {
                        dnew[2 * tid] = app;
                        dnew[2 * tid + 1] = aqq;
                    }
                } else {
                    p = q = -1;
                }
                pp[tid] = p; qq[tid] = q; cs[tid] = c; ss[tid] = s; eph[tid] = ph;
            }
            __syncthreads();
            // 2. column pass M <- M G and U <- U G
            for (int e = tid; e < N * half; e += nt) {
                int i = e / half, j = e % half;
                int p = pp[j], q = qq[j];
                if (p < 0) continue;
                T c = cs[j], s = ss[j];
                cplx<T> ph = eph[j];
                cplx<T> xp = M[i * ld + p], xq = M[i * ld + q];
                // X'[i][p] = c xp - s e^{-i phi} xq ; X'[i][q] = s e^{i phi} xp + c xq
                M[i * ld + p] = c * xp - s * mul_cj(xq, ph);
                M[i * ld + q] = s * (ph * xp) + c * xq;
                cplx<T> vp = Vv[i * ld + p], vq = Vv[i * ld + q];
                Vv[i * ld + p] = c * vp - s * mul_cj(vq, ph);
                Vv[i * ld + q] = s * (ph * vp) + c * vq;
            }
            __syncthreads();
            // 3. row pass M <- G^dag M
            for (int e = tid; e < N * half; e += nt) {
                int i = e / half, j = e % half;
                int p = pp[j], q = qq[j];
                if (p < 0) continue;
                T c = cs[j], s = ss[j];
                cplx<T> ph = eph[j];
                cplx<T> xp = M[p * ld + i], xq = M[q * ld + i];
                // X'[p][i] = c xp - s e^{i phi} xq ; X'[q][i] = s e^{-i phi} xp + c xq
                M[p * ld + i] = c * xp - s * (ph * xq);
                M[q * ld + i] = s * mul_cj(xp, ph) + c * xq;
            }
            __syncthreads();
            // 4. exact 2x2 result on the rotated pairs
            if (tid < half) {
                int p = pp[tid], q = qq[tid];
                if (p >= 0) {
                    M[p * ld + p] = mk(dnew[2 * tid], (T)0);
                    M[q * ld + q] = mk(dnew[2 * tid + 1], (T)0);
                    M[p * ld + q] = mk((T)0, (T)0);
                    M[q * ld + p] = mk((T)0, (T)0);
                }
            }
            __syncthreads();
        }
        // convergence: off-diagonal norm
        T off = 0;
        for (int e = tid; e < NN; e += nt) {
            int i = e / N, j = e % N;
            if (i != j) off += abs2(M[i * ld + j]);
        }
        red[tid] = off;
        __syncthreads();
        for (int w = nt / 2; w > 0; w >>= 1) {
            if (tid < w) red[tid] += red[tid + w];
            __syncthreads();
        }
        if (tid == 0) s_conv = (red[0] <= tol2) ? 1 : 0;
        __syncthreads();
        converged = s_conv != 0;
        __syncthreads();
    }
    if (tid == 0) {
        atomicMax(sweeps_max, sweep);
        if (!converged) atomicAdd(flag_cap, 1);
    }
    // sort ascending (stable on ties) and write E, U
    T* dg = red;  // reuse: diagonal values
    for (int i = tid; i < N; i += nt) dg[i] = M[i * ld + i].re;
    __syncthreads();
    for (int i = tid; i < N; i += nt) {
        T ei = dg[i];
        int rank = 0;
        for (int j = 0; j < N; ++j) {
            T ej = dg[j];
            rank += (ej < ei || (ej == ei && j < i)) ? 1 : 0;
        }
        E[(size_t)k * N + rank] = ei;
        for (int row = 0; row < N; ++row) U[(size_t)k * NN + row * N + rank] = Vv[row * ld + i];
    }
    if (redo_flag) {
        __syncthreads();
        if (tid == 0) {
            // smallest gap between any two eigenvalues (sorted neighbours)
            T mingap = (T)1e30;
            for (int i = 0; i < N; ++i)
                for (int j = i + 1; j < N; ++j) {
                    T d = fabs(dg[i] - dg[j]);
                    mingap = d < mingap ? d : mingap;
                }
            redo_flag[k] = (!converged || (double)mingap < degen_gap || !(mingap == mingap)) ? 1 : 0;
        }
    }
}

}  // namespace

template <typename T>
size_t eig_smem_bytes(int N) {
    const int ld = N + 1;
    size_t b = 2 * (size_t)N * ld * sizeof(cplx<T>);
    b += 2 * (kMaxN / 2) * sizeof(T) + (kMaxN / 2) * sizeof(cplx<T>) + kMaxN * sizeof(T);
    b += 2 * (kMaxN / 2) * sizeof(int) + 256 * sizeof(T);
    return (b + 15) & ~(size_t)15;
}

template <typename T>
cudaError_t launch_eig(int N, int64_t nk, const cplx<T>* W, int nbW, T* E, cplx<T>* U, int max_sweeps,
                       int* sweeps_max, int* flag_cap, double degen_gap, int* redo_flag, cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    size_t smem = eig_smem_bytes<T>(N);
    cudaError_t e = cudaFuncSetAttribute(jacobi_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int threads = N <= 16 ? 128 : 256;
    jacobi_kernel<T><<<(unsigned)nk, threads, smem, s>>>(N, W, nbW, E, U, max_sweeps, sweeps_max, flag_cap, degen_gap,
                                                         redo_flag);
    return cudaGetLastError();
}

template cudaError_t launch_eig<double>(int, int64_t, const cplx<double>*, int, double*, cplx<double>*, int, int*, int*,
                                        double, int*, cudaStream_t);
template cudaError_t launch_eig<float>(int, int64_t, const cplx<float>*, int, float*, cplx<float>*, int, int*, int*,
                                       double, int*, cudaStream_t);

}  // namespace mepi
