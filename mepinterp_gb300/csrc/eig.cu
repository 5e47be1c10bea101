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

// FP64 refinement of the FP32 eigenpairs (U, lambda) against the FP64 H(k),
// in residual form so that a single product runs in FP64:
//   R = H U - U diag(lambda)                 FP64 (the only cancelling product)
//   P = U^dag R                              FP32 (R is small: its rounding is
//                                            relative to |R|, not to |H|)
//   rho_n = lambda_n + P_nn / S_nn,  S_nn = |u_n|^2      (normalised Rayleigh
//                                            quotient, FP64)
//   E_n = rho_n + sum_{m!=n} |P_mn|^2 / (rho_n - rho_m)  (second order)
//   C_mn = P_mn / (rho_n - rho_m),  U' = (U + U C) diag(S_nn)^-1/2    (FP32)
// C fixes both the eigenvector error and the loss of orthogonality of the
// warm-started FP32 vectors to first order: <u'_m|u'_n> = S_mn + C_mn +
// conj(C_nm) + O(2nd) = O(2nd).  The energies are then exact to third order
// in |P| / gap and the vectors to second order, for any gap above degen_gap.
// A k-point with a gap at or below degen_gap, an unconverged FP32 Jacobi run
// (flag already set) or non-finite values is flagged for the full FP64 rerun.
// Eigenpairs are re-sorted by the refined energies.
__global__ void __launch_bounds__(256) refine_kernel(int N, const cplx<double>* __restrict__ H64,
                                                     const float* __restrict__ lam, cplx<float>* __restrict__ U,
                                                     double* __restrict__ E64, double degen_gap,
                                                     int* __restrict__ redo_flag) {
    extern __shared__ unsigned char smem_raw[];
    const int Np = N + (N & 1), NPP = Np * Np, h = Np / 2;
    cplx<double>* Hs = reinterpret_cast<cplx<double>*>(smem_raw);
    double* rho = reinterpret_cast<double*>(Hs + NPP);
    double* En = rho + Np;
    double* Sn = En + Np;
    cplx<float>* Us = reinterpret_cast<cplx<float>*>(Sn + Np);
    cplx<float>* Rs = Us + NPP;
    cplx<float>* Ps = Rs + NPP;
    __shared__ float ls[kMaxN];
    __shared__ int s_flag;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int64_t k = blockIdx.x;
    const int NN = N * N;
    for (int e = tid; e < NPP; e += nt) {
        const int i = e / Np, j = e % Np;
        cplx<double> hv = mk(0.0, 0.0);
        cplx<float> uv = mk(0.f, 0.f);
        if (i < N && j < N) {
            const int a = i < j ? i : j, b = i < j ? j : i;
            const cplx<double> x = H64[(size_t)k * NN + a * N + b];
            hv = (i < j) ? x : (i > j) ? conjg(x) : mk(x.re, 0.0);
            uv = U[(size_t)k * NN + i * N + j];
        }
        Hs[e] = hv;
        Us[e] = uv;
    }
    for (int n = tid; n < Np; n += nt) ls[n] = n < N ? lam[(size_t)k * N + n] : 0.f;
    if (tid == 0) s_flag = redo_flag ? redo_flag[k] : 0;
    __syncthreads();
    // R = H U - U diag(lambda): FP64 accumulation, 2 x 2 tiles per thread
    for (int t = tid; t < h * h; t += nt) {
        const int i = 2 * (t / h), c = 2 * (t % h);
        cplx<double> a00 = mk(0.0, 0.0), a01 = a00, a10 = a00, a11 = a00;
        for (int l = 0; l < Np; ++l) {
            const cplx<double> h0 = Hs[i * Np + l], h1 = Hs[(i + 1) * Np + l];
            const cplx<float> u0f = Us[l * Np + c], u1f = Us[l * Np + c + 1];
            const cplx<double> u0 = mk((double)u0f.re, (double)u0f.im), u1 = mk((double)u1f.re, (double)u1f.im);
            fma_c(a00, h0, u0);
            fma_c(a01, h0, u1);
            fma_c(a10, h1, u0);
            fma_c(a11, h1, u1);
        }
        const double l0 = ls[c], l1 = ls[c + 1];
        auto res = [&](cplx<double> acc, int r, int col, double lv) {
            const cplx<float> u = Us[r * Np + col];
            Rs[r * Np + col] = mk((float)(acc.re - lv * (double)u.re), (float)(acc.im - lv * (double)u.im));
        };
        res(a00, i, c, l0);
        res(a01, i, c + 1, l1);
        res(a10, i + 1, c, l0);
        res(a11, i + 1, c + 1, l1);
    }
    __syncthreads();
    // P = U^dag R (FP32)
    smem_cgemm<float, true>(Np, Np, Us, Rs, Ps, tid, nt);
    for (int n = tid; n < N; n += nt) {
        double s = 0.0;
        for (int l = 0; l < N; ++l) {
            const cplx<float> u = Us[l * Np + n];
            s += (double)u.re * u.re + (double)u.im * u.im;
        }
        Sn[n] = s;
    }
    __syncthreads();
    for (int n = tid; n < N; n += nt) rho[n] = (double)ls[n] + (double)Ps[n * Np + n].re / Sn[n];
    __syncthreads();
    for (int n = tid; n < N; n += nt) {
        double e2 = rho[n];
        bool bad = !isfinite(e2);
        for (int m = 0; m < N; ++m) {
            if (m == n) continue;
            const double d = rho[n] - rho[m];
            if (!(fabs(d) > degen_gap)) { bad = true; continue; }
            const cplx<float> p = Ps[m * Np + n];
            e2 += ((double)p.re * p.re + (double)p.im * p.im) / d;
        }
        En[n] = e2;
        if (bad || !isfinite(e2)) s_flag = 1;
    }
    __syncthreads();
    // C in place of P (zero diagonal and zero for flagged gaps)
    for (int e = tid; e < NPP; e += nt) {
        const int m = e / Np, n = e % Np;
        cplx<float> c = mk(0.f, 0.f);
        if (m < N && n < N && m != n) {
            const double d = rho[n] - rho[m];
            if (fabs(d) > degen_gap) c = mk((float)((double)Ps[e].re / d), (float)((double)Ps[e].im / d));
        }
        Ps[e] = c;
    }
    __syncthreads();
    // U' = U + U C (FP32) into Rs
    smem_cgemm<float, false>(Np, Np, Us, Ps, Rs, tid, nt);
    __syncthreads();
    for (int n = tid; n < N; n += nt) {
        const double en = En[n];
        int rank = 0;
        for (int j = 0; j < N; ++j) rank += (En[j] < en || (En[j] == en && j < n)) ? 1 : 0;
        E64[(size_t)k * N + rank] = en;
        const float sc = (float)(1.0 / sqrt(Sn[n]));
        for (int row = 0; row < N; ++row) {
            const cplx<float> u = Us[row * Np + n] + Rs[row * Np + n];
            U[(size_t)k * NN + row * N + rank] = mk(u.re * sc, u.im * sc);
        }
    }
    __syncthreads();
    if (tid == 0 && redo_flag) redo_flag[k] = s_flag ? 1 : 0;
}

size_t refine_smem_bytes(int N) {
    const size_t Np = N + (N & 1);
    return Np * Np * sizeof(cplx<double>) + 3 * Np * sizeof(double) + 3 * Np * Np * sizeof(cplx<float>);
}

cudaError_t launch_refine(int N, int64_t nk, const cplx<double>* H64, const float* lam, cplx<float>* U, double* E64,
                          double degen_gap, int* redo_flag, cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    const size_t smem = refine_smem_bytes(N);
    cudaError_t e = cudaFuncSetAttribute(refine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    refine_kernel<<<(unsigned)nk, N <= 16 ? 128 : 256, smem, s>>>(N, H64, lam, U, E64, degen_gap, redo_flag);
    return cudaGetLastError();
}

template cudaError_t launch_eig<double>(int, int64_t, const cplx<double>*, int, const cplx<double>*, double*,
                                        cplx<double>*, int, int*, int*, double, int*, cudaStream_t);
template cudaError_t launch_eig<float>(int, int64_t, const cplx<float>*, int, const cplx<double>*, float*,
                                       cplx<float>*, int, int*, int*, double, int*, cudaStream_t);

}  // namespace mepi
