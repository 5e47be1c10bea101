// Batched Hermitian eigensolver replacing zheevd_wrapper
// (src/matrix_math.f90:192-226: jobz='V', uplo='U', eigenvalues ascending,
// eigenvectors in the columns of U).
//
// A CTA diagonalises a run of consecutive k-points (adjacent along kx): the
// first from the identity, each next one warm-started from its neighbour's
// eigenvectors V as V^dag H V, which typically needs a few sweeps instead of
// six or seven.  The matrix and the eigenvector accumulator live in shared
// memory; each sweep of the two-sided cyclic Jacobi method runs as N-1
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
__global__ void __launch_bounds__(256) jacobi_kernel(int N, int64_t nk, int kblock, const cplx<T>* __restrict__ W,
                                                     int nbW, const cplx<double>* __restrict__ H64,
                                                     T* __restrict__ E, cplx<T>* __restrict__ U, int max_sweeps,
                                                     int* sweeps_max, int* flag_cap, double degen_gap,
                                                     int* redo_flag) {
    extern __shared__ unsigned char smem_raw[];
    const int ld = N + 1;                       // padded row stride
    cplx<T>* M = reinterpret_cast<cplx<T>*>(smem_raw);
    cplx<T>* Vv = M + N * ld;                   // eigenvector accumulator
    cplx<T>* Ts = Vv + N * ld;                  // warm-start product / sorted copy
    T* cs = reinterpret_cast<T*>(Ts + N * ld);  // per pair: c, s
    T* ss = cs + kMaxN / 2;
    cplx<T>* eph = reinterpret_cast<cplx<T>*>(ss + kMaxN / 2);  // e^{i phi}
    T* dnew = reinterpret_cast<T*>(eph + kMaxN / 2);           // new diagonal (2 per pair)
    int* pp = reinterpret_cast<int*>(dnew + kMaxN);
    int* qq = pp + kMaxN / 2;
    T* red = reinterpret_cast<T*>(qq + kMaxN / 2);            // reduction scratch [256]
    __shared__ int s_conv;

    const int tid = threadIdx.x, nt = blockDim.x;
    const int NN = N * N;
    const int Np = N + (N & 1);
    const int half = Np / 2;
    const int Np1 = Np - 1;

    for (int jb = 0; jb < kblock; ++jb) {
        const int64_t k = (int64_t)blockIdx.x * kblock + jb;
        if (k >= nk) break;
        const bool warm = jb > 0;   // Vv holds the previous k-point's sorted eigenvectors
        __syncthreads();
        // load (from the FP64 H(k) when given), Hermitise from the upper triangle
        for (int e = tid; e < NN; e += nt) {
            int i = e / N, j = e % N;
            int a = i < j ? i : j, b = i < j ? j : i;
            cplx<T> h;
            if (H64) {
                const cplx<double> x = H64[(size_t)k * NN + a * N + b];
                h = mk((T)x.re, (T)x.im);
            } else {
                h = W[(size_t)k * nbW * NN + a * N + b];
            }
            cplx<T> v = (i < j) ? h : (i > j) ? conjg(h) : mk(h.re, (T)0);
            M[i * ld + j] = v;
            if (!warm) Vv[i * ld + j] = mk((T)(i == j ? 1 : 0), (T)0);
        }
        // ||H||_F^2 (unchanged by the unitary warm start)
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
        if (warm) {
            // M <- V^dag H V with V the previous eigenvectors (neighbouring k)
            if ((N & 1) == 0) {
                smem_cgemm<T, false>(N, ld, M, Vv, Ts, tid, nt);
                __syncthreads();
                smem_cgemm<T, true>(N, ld, Vv, Ts, M, tid, nt);
            } else {
                for (int e = tid; e < NN; e += nt) {
                    int i = e / N, c = e % N;
                    cplx<T> acc = mk((T)0, (T)0);
                    for (int l = 0; l < N; ++l) fma_c(acc, M[i * ld + l], Vv[l * ld + c]);
                    Ts[i * ld + c] = acc;
                }
                __syncthreads();
                for (int e = tid; e < NN; e += nt) {
                    int i = e / N, c = e % N;
                    cplx<T> acc = mk((T)0, (T)0);
                    for (int l = 0; l < N; ++l) fma_cjc(acc, Vv[l * ld + i], Ts[l * ld + c]);
                    M[i * ld + c] = acc;
                }
            }
            __syncthreads();
            // restore exact Hermiticity of the rotated matrix
            for (int e = tid; e < NN; e += nt) {
                int i = e / N, j = e % N;
                if (i < j) {
                    cplx<T> x = M[i * ld + j], y = M[j * ld + i];
                    cplx<T> h = mk((T)0.5 * (x.re + y.re), (T)0.5 * (x.im - y.im));
                    Ts[i * ld + j] = h;
                    Ts[j * ld + i] = conjg(h);
                } else if (i == j) {
                    Ts[i * ld + i] = mk(M[i * ld + i].re, (T)0);
                }
            }
            __syncthreads();
            for (int e = tid; e < NN; e += nt) {
                int i = e / N, j = e % N;
                M[i * ld + j] = Ts[i * ld + j];
            }
            __syncthreads();
        }

        const T tolr = (T)(4.0 * EigTol<T>::eps) * sqrt((T)N);
        const T tol2 = tolr * tolr * fro2;
        const T gskip = (T)EigTol<T>::skip * sqrt(fro2);
        int sweep = 0;
        bool converged = (N == 1);
        // a warm start may already be converged: test before the first sweep
        if (warm) {
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
                // 2. column pass M <- M G and U <- U G (consecutive threads walk the
                //    rows of one pair: padded rows put them in distinct banks)
                for (int e = tid; e < N * half; e += nt) {
                    int j = e / N, i = e % N;
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
                // 3. row pass M <- G^dag M (consecutive threads walk one row)
                for (int e = tid; e < N * half; e += nt) {
                    int j = e / N, i = e % N;
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
        // sort ascending (stable on ties), write E and U, keep the sorted
        // eigenvectors in Vv as the next k-point's warm start
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
            for (int row = 0; row < N; ++row) {
                const cplx<T> v = Vv[row * ld + i];
                U[(size_t)k * NN + row * N + rank] = v;
                Ts[row * ld + rank] = v;
            }
        }
        __syncthreads();
        if (redo_flag && tid == 0) {
            // smallest gap between any two eigenvalues
            T mingap = (T)1e30;
            for (int i = 0; i < N; ++i)
                for (int j = i + 1; j < N; ++j) {
                    T d = fabs(dg[i] - dg[j]);
                    mingap = d < mingap ? d : mingap;
                }
            redo_flag[k] = (!converged || (double)mingap < degen_gap || !(mingap == mingap)) ? 1 : 0;
        }
        for (int e = tid; e < NN; e += nt) {
            int i = e / N, j = e % N;
            Vv[i * ld + j] = Ts[i * ld + j];
        }
    }
}

}  // namespace

template <typename T>
size_t eig_smem_bytes(int N) {
    const int ld = N + 1;
    size_t b = 3 * (size_t)N * ld * sizeof(cplx<T>);
    b += 2 * (kMaxN / 2) * sizeof(T) + (kMaxN / 2) * sizeof(cplx<T>) + kMaxN * sizeof(T);
    b += 2 * (kMaxN / 2) * sizeof(int) + 256 * sizeof(T);
    return (b + 15) & ~(size_t)15;
}

template <typename T>
cudaError_t launch_eig(int N, int64_t nk, const cplx<T>* W, int nbW, const cplx<double>* H64, T* E, cplx<T>* U,
                       int max_sweeps, int* sweeps_max, int* flag_cap, double degen_gap, int* redo_flag,
                       cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    size_t smem = eig_smem_bytes<T>(N);
    cudaError_t e = cudaFuncSetAttribute(jacobi_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int threads = N <= 16 ? 128 : 256;
    // a run of consecutive k-points per CTA, each warm-started from its
    // neighbour's eigenvectors (consecutive k are adjacent along kx)
    const int kblock = 8;
    const unsigned grid = (unsigned)((nk + kblock - 1) / kblock);
    jacobi_kernel<T><<<grid, threads, smem, s>>>(N, nk, kblock, W, nbW, H64, E, U, max_sweeps, sweeps_max, flag_cap,
                                                 degen_gap, redo_flag);
    return cudaGetLastError();
}

// FP64 refinement of FP32 eigenpairs against the FP64 H(k):
//   T = H U, H' = U^dag T (both FP64), E_n = Re H'_nn (Rayleigh quotients, whose
//   error is second order in the FP32 eigenvector error), and, when first_order
//   is set, U <- U (1 + X) with X_mn = H'_mn / (E_n - E_m) for the pairs whose
//   gap exceeds degen_gap.  A k-point with a gap at or below degen_gap, or with
//   non-finite values, is flagged for the full FP64 rerun.  Eigenpairs are
//   re-sorted by the refined energies.
__global__ void __launch_bounds__(256) refine_kernel(int N, const cplx<double>* __restrict__ H64,
                                                     cplx<float>* __restrict__ U, double* __restrict__ E64,
                                                     double degen_gap, int first_order, int* __restrict__ redo_flag) {
    extern __shared__ unsigned char smem_raw[];
    const int NN = N * N;
    cplx<double>* Hs = reinterpret_cast<cplx<double>*>(smem_raw);
    cplx<double>* Us = Hs + NN;
    cplx<double>* Ts = Us + NN;
    double* Ev = reinterpret_cast<double*>(Ts + NN);
    __shared__ int s_flag;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int64_t k = blockIdx.x;
    for (int e = tid; e < NN; e += nt) {
        int i = e / N, j = e % N;
        int a = i < j ? i : j, b = i < j ? j : i;
        cplx<double> h = H64[(size_t)k * NN + a * N + b];
        Hs[e] = (i < j) ? h : (i > j) ? conjg(h) : mk(h.re, 0.0);
        const cplx<float> u = U[(size_t)k * NN + e];
        Us[e] = mk((double)u.re, (double)u.im);
    }
    if (tid == 0) s_flag = redo_flag ? redo_flag[k] : 0;
    __syncthreads();
    // T = H U
    for (int e = tid; e < NN; e += nt) {
        int i = e / N, c = e % N;
        cplx<double> acc = mk(0.0, 0.0);
        for (int l = 0; l < N; ++l) fma_c(acc, Hs[i * N + l], Us[l * N + c]);
        Ts[e] = acc;
    }
    __syncthreads();
    // H' = U^dag T  (into Hs)
    for (int e = tid; e < NN; e += nt) {
        int i = e / N, c = e % N;
        cplx<double> acc = mk(0.0, 0.0);
        for (int l = 0; l < N; ++l) fma_cjc(acc, Us[l * N + i], Ts[l * N + c]);
        Hs[e] = acc;
    }
    __syncthreads();
    for (int n = tid; n < N; n += nt) Ev[n] = Hs[n * N + n].re;
    __syncthreads();
    // flag near degeneracies (and non-finite energies)
    for (int e = tid; e < NN; e += nt) {
        int i = e / N, j = e % N;
        if (i < j && !(fabs(Ev[i] - Ev[j]) > degen_gap)) s_flag = 1;
    }
    if (first_order) {
        // X into Ts, then U' = U + U X into Hs
        for (int e = tid; e < NN; e += nt) {
            int m = e / N, n = e % N;
            const double d = Ev[n] - Ev[m];
            Ts[e] = (m != n && fabs(d) > degen_gap) ? mk(Hs[e].re / d, Hs[e].im / d) : mk(0.0, 0.0);
        }
        __syncthreads();
        for (int e = tid; e < NN; e += nt) {
            int i = e / N, n = e % N;
            cplx<double> acc = Us[e];
            for (int m = 0; m < N; ++m) fma_c(acc, Us[i * N + m], Ts[m * N + n]);
            Hs[e] = acc;
        }
        __syncthreads();
        for (int e = tid; e < NN; e += nt) Us[e] = Hs[e];
    }
    __syncthreads();
    for (int n = tid; n < N; n += nt) {
        const double en = Ev[n];
        int rank = 0;
        for (int j = 0; j < N; ++j) rank += (Ev[j] < en || (Ev[j] == en && j < n)) ? 1 : 0;
        E64[(size_t)k * N + rank] = en;
        for (int row = 0; row < N; ++row) {
            const cplx<double> u = Us[row * N + n];
            U[(size_t)k * NN + row * N + rank] = mk((float)u.re, (float)u.im);
        }
        if (!isfinite(en)) s_flag = 1;
    }
    __syncthreads();
    if (tid == 0 && redo_flag) redo_flag[k] = s_flag ? 1 : 0;
}

// Mixed form without the FP64 refinement: flag the k-points whose result
// could flip under the FP32 eigenvalue error -- a Niu term whose product
// denominator |(E0-En)^2 (E0-Em)| lies within a relative mask_eps of kuboTol
// (src/mep_niu.f90:72-73, :131-132), or, for the T = 0 step occupation, a band
// within fermi_eps of a Fermi energy -- for the FP64 rerun, and hand the FP32
// energies on as FP64.
__global__ void __launch_bounds__(128) window_flag_kernel(int N, const float* __restrict__ E32, double* __restrict__ E64,
                                                          int nval, float tol, float mask_eps, int nE,
                                                          const double* __restrict__ ef, int step_occ,
                                                          double fermi_eps, int* __restrict__ flags) {
    __shared__ float Es[kMaxN];
    __shared__ int hit;
    const int64_t k = blockIdx.x;
    const int tid = threadIdx.x, NN = N * N;
    if (tid == 0) hit = 0;
    for (int n = tid; n < N; n += blockDim.x) {
        const float e = E32[(size_t)k * N + n];
        Es[n] = e;
        E64[(size_t)k * N + n] = (double)e;
    }
    __syncthreads();
    int h = 0;
    if (flags) {
        const float lo = tol * (1.f - mask_eps), hi = tol * (1.f + mask_eps);
        for (int t = tid; t < nval * NN; t += blockDim.x) {
            const int n0 = t / NN, n = (t / N) % N, m = t % N;
            if (n == n0 || m == n0) continue;
            const float d0n = Es[n0] - Es[n], d0m = Es[n0] - Es[m];
            const float den = fabsf(d0n * d0n * d0m);
            h |= (den >= lo && den <= hi) ? 1 : 0;
        }
        if (step_occ)
            for (int t = tid; t < N * nE; t += blockDim.x) {
                const int n = t / nE, e = t % nE;
                h |= (fabs((double)Es[n] - ef[e]) < fermi_eps) ? 1 : 0;
            }
        if (h) atomicOr(&hit, 1);
    }
    __syncthreads();
    if (flags && tid == 0 && hit) flags[k] = 1;
}

cudaError_t launch_window_flags(int N, int64_t nk, const float* E32, double* E64, int nval, double tol, double mask_eps,
                                int nE, const double* ef, int step_occ, double fermi_eps, int* flags, cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    window_flag_kernel<<<(unsigned)nk, 128, 0, s>>>(N, E32, E64, nval, (float)tol, (float)mask_eps, nE, ef, step_occ,
                                                    fermi_eps, flags);
    return cudaGetLastError();
}

cudaError_t launch_refine(int N, int64_t nk, const cplx<double>* H64, cplx<float>* U, double* E64, double degen_gap,
                          int first_order, int* redo_flag, cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    const size_t smem = 3 * (size_t)N * N * sizeof(cplx<double>) + (size_t)N * sizeof(double);
    cudaError_t e = cudaFuncSetAttribute(refine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    refine_kernel<<<(unsigned)nk, N <= 16 ? 128 : 256, smem, s>>>(N, H64, U, E64, degen_gap, first_order, redo_flag);
    return cudaGetLastError();
}

template cudaError_t launch_eig<double>(int, int64_t, const cplx<double>*, int, const cplx<double>*, double*,
                                        cplx<double>*, int, int*, int*, double, int*, cudaStream_t);
template cudaError_t launch_eig<float>(int, int64_t, const cplx<float>*, int, const cplx<double>*, float*,
                                       cplx<float>*, int, int*, int*, double, int*, cudaStream_t);

}  // namespace mepi
