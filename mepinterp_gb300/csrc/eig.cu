// Batched Hermitian eigensolver replacing zheevd_wrapper
// (src/matrix_math.f90:192-226: jobz='V', uplo='U', eigenvalues ascending,
// eigenvectors in the columns of U).
//
// A CTA diagonalises a run of consecutive k-points of the run's order (mesh
// neighbours along kz within a (qx, qy) column for the separable sums): the
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

__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Stop when ||offdiag(M)||_F <= 4 sqrt(N) eps ||H||_F (the rounding floor of the
// off-diagonal entries); rotations with |M_pq| below skip * ||H||_F are skipped
// (their phase e^{i phi} would not be unitary to working precision).
template <typename T> struct EigTol;
template <> struct EigTol<double> { static constexpr double eps = 2.220446049250313e-16, skip = 1e-20; };
template <> struct EigTol<float> { static constexpr double eps = 1.1920928955078125e-07, skip = 1e-10; };

// Sum over the CTA (256 threads or fewer, a multiple of 32).
template <typename T>
__device__ __forceinline__ T cta_sum(T v, T* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[w] = v;
    __syncthreads();
    T s = 0;
    for (int i = 0; i < nw; ++i) s += red[i];
    return s;
}

// Rotation of one pair of a round, packed so that a thread fetches it with
// one vector load (c, s, e^{i phi}) plus one for the indices.
template <typename T>
struct alignas(4 * sizeof(T)) RotPar {
    T c, s, pr, pi;
};

// One CTA diagonalises a run of kblock consecutive k-points.  The matrix M
// and the eigenvector accumulator V live in shared memory as separate real
// and imaginary planes with row stride NP + 1 (NP = the band count padded to
// a power of two; padded rows and columns hold zeros in M and the identity
// in V, and the pairs that touch them are never rotated).  A round of the
// round-robin ordering rotates NP/2 disjoint pairs at once; because the pairs
// partition the indices, M <- G^dag M G splits into independent 2 x 2 blocks
// (rows of pair A, columns of pair B), Z = G_A^dag X G_B, which each thread
// updates in place -- one pass and two barriers per round.
template <typename T, int NP>
__global__ void __launch_bounds__(256) jacobi_kernel(int N, int64_t nk, int kblock, const cplx<T>* __restrict__ W,
                                                     int nbW, const float4* __restrict__ Hdf,
                                                     T* __restrict__ E, cplx<T>* __restrict__ U, int max_sweeps,
                                                     int* sweeps_max, int* flag_cap, double degen_gap,
                                                     int* redo_flag, float gap_theta) {
    constexpr int HP = NP / 2, LD = NP + 1, PL = NP * LD;
    extern __shared__ unsigned char smem_raw[];
    T* Mr = reinterpret_cast<T*>(smem_raw);
    T* Mi = Mr + PL;
    T* Vr = Mi + PL;
    T* Vi = Vr + PL;
    T* Tr = Vi + PL;  // warm-start product / sorted eigenvectors
    T* Ti = Tr + PL;
    __shared__ RotPar<T> s_rot[HP];
    __shared__ int2 s_pq[HP];
    __shared__ T s_d0[HP], s_d1[HP];
    __shared__ int s_fix[HP];
    __shared__ T red[8];
    __shared__ T s_E[NP];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int NN = N * N;

    for (int jb = 0; jb < kblock; ++jb) {
        const int64_t k = (int64_t)blockIdx.x * kblock + jb;
        if (k >= nk) break;
        const bool warm = jb > 0;   // V holds the previous k-point's sorted eigenvectors
        __syncthreads();
        // load (from the FP64 H(k) when given), Hermitise from the upper triangle
        T part = 0;
        for (int e = tid; e < NP * NP; e += nt) {
            const int i = e / NP, j = e % NP;
            cplx<T> v = mk((T)0, (T)0);
            if (i < N && j < N) {
                const int a = i < j ? i : j, b = i < j ? j : i;
                cplx<T> h;
                if (Hdf) {
                    const float4 x = Hdf[(size_t)k * NN + a * N + b];
                    h = mk((T)x.x, (T)x.y);
                } else {
                    h = W[(size_t)k * nbW * NN + a * N + b];
                }
                v = (i < j) ? h : (i > j) ? conjg(h) : mk(h.re, (T)0);
            }
            Mr[i * LD + j] = v.re;
            Mi[i * LD + j] = v.im;
            part += abs2(v);
            if (!warm) {
                Vr[i * LD + j] = (T)(i == j ? 1 : 0);
                Vi[i * LD + j] = (T)0;
            }
        }
        const T fro2 = cta_sum(part, red);   // ||H||_F^2, unchanged by the unitary warm start
        if (warm) {
            // T = M V, then M = V^dag T (2 x 2 output tiles per thread)
            for (int t = tid; t < HP * HP; t += nt) {
                const int i = 2 * (t / HP), j = 2 * (t % HP);
                cplx<T> c00 = mk((T)0, (T)0), c01 = c00, c10 = c00, c11 = c00;
                for (int l = 0; l < NP; ++l) {
                    const cplx<T> a0 = mk(Mr[i * LD + l], Mi[i * LD + l]), a1 = mk(Mr[(i + 1) * LD + l], Mi[(i + 1) * LD + l]);
                    const cplx<T> b0 = mk(Vr[l * LD + j], Vi[l * LD + j]), b1 = mk(Vr[l * LD + j + 1], Vi[l * LD + j + 1]);
                    fma_c(c00, a0, b0); fma_c(c01, a0, b1); fma_c(c10, a1, b0); fma_c(c11, a1, b1);
                }
                Tr[i * LD + j] = c00.re; Ti[i * LD + j] = c00.im;
                Tr[i * LD + j + 1] = c01.re; Ti[i * LD + j + 1] = c01.im;
                Tr[(i + 1) * LD + j] = c10.re; Ti[(i + 1) * LD + j] = c10.im;
                Tr[(i + 1) * LD + j + 1] = c11.re; Ti[(i + 1) * LD + j + 1] = c11.im;
            }
            __syncthreads();
            for (int t = tid; t < HP * HP; t += nt) {
                const int i = 2 * (t / HP), j = 2 * (t % HP);
                cplx<T> c00 = mk((T)0, (T)0), c01 = c00, c10 = c00, c11 = c00;
                for (int l = 0; l < NP; ++l) {
                    const cplx<T> a0 = conjg(mk(Vr[l * LD + i], Vi[l * LD + i]));
                    const cplx<T> a1 = conjg(mk(Vr[l * LD + i + 1], Vi[l * LD + i + 1]));
                    const cplx<T> b0 = mk(Tr[l * LD + j], Ti[l * LD + j]), b1 = mk(Tr[l * LD + j + 1], Ti[l * LD + j + 1]);
                    fma_c(c00, a0, b0); fma_c(c01, a0, b1); fma_c(c10, a1, b0); fma_c(c11, a1, b1);
                }
                Mr[i * LD + j] = c00.re; Mi[i * LD + j] = c00.im;
                Mr[i * LD + j + 1] = c01.re; Mi[i * LD + j + 1] = c01.im;
                Mr[(i + 1) * LD + j] = c10.re; Mi[(i + 1) * LD + j] = c10.im;
                Mr[(i + 1) * LD + j + 1] = c11.re; Mi[(i + 1) * LD + j + 1] = c11.im;
            }
            __syncthreads();
            // restore exact Hermiticity of the rotated matrix
            for (int e = tid; e < NP * NP; e += nt) {
                const int i = e / NP, j = e % NP;
                if (i < j) {
                    const T re = (T)0.5 * (Mr[i * LD + j] + Mr[j * LD + i]);
                    const T im = (T)0.5 * (Mi[i * LD + j] - Mi[j * LD + i]);
                    Mr[i * LD + j] = re; Mi[i * LD + j] = im;
                    Mr[j * LD + i] = re; Mi[j * LD + i] = -im;
                } else if (i == j) {
                    Mi[i * LD + i] = (T)0;
                }
            }
            __syncthreads();
        }

        const T tolr = (T)(4.0 * EigTol<T>::eps) * sqrt((T)N);
        const T tol2 = tolr * tolr * fro2;
        const T gskip = (T)EigTol<T>::skip * sqrt(fro2);
        auto off_norm = [&]() {
            T o = 0;
            for (int e = tid; e < NP * NP; e += nt) {
                const int i = e / NP, j = e % NP;
                if (i != j) o += Mr[i * LD + j] * Mr[i * LD + j] + Mi[i * LD + j] * Mi[i * LD + j];
            }
            return cta_sum(o, red);
        };
        // With gap_theta > 0 (the FP32 form, whose eigenpairs the FP64 residual
        // refinement finishes to second order), a pair is rotated only while
        // |M_pq| > gap_theta |M_pp - M_qq|: the refinement's error is then of
        // order gap_theta^3.  Rounds in which no pair rotates are skipped, and
        // a sweep without rotations ends the run.
        const T gth = (T)gap_theta;
        auto strong = [&](int p, int q) {
            const T xr = Mr[p * LD + q], xi = Mi[p * LD + q];
            const T g = sqrt(xr * xr + xi * xi);
            return g > gskip && !(gth > (T)0 && g <= gth * fabs(Mr[q * LD + q] - Mr[p * LD + p]));
        };
        int sweep = 0;
        // a warm start may already be converged: test before the first sweep
        bool converged = (N == 1) || (warm && off_norm() <= tol2);
        if (!converged && warm && gth > (T)0) {
            int any = 0;
            for (int e = tid; e < N * N; e += nt) {
                const int i = e / N, j = e % N;
                if (i < j && strong(i, j)) any = 1;
            }
            converged = !__syncthreads_or(any);
        }
        for (sweep = 0; sweep < max_sweeps && !converged; ++sweep) {
            int rotated = 0;
            for (int r = 0; r < NP - 1; ++r) {
                // 1. rotation parameters of the pairs of this round
                if (tid < HP) {
                    const int a = tid == 0 ? NP - 1 : (r + tid) % (NP - 1);
                    const int b = tid == 0 ? r : (r - tid + NP - 1) % (NP - 1);
                    const int p = a < b ? a : b, q = a < b ? b : a;
                    T c = 1, sn = 0, pr = 1, pi = 0, d0 = 0, d1 = 0;
                    int fix = 0;
                    if (q < N) {
                        const T app = Mr[p * LD + p], aqq = Mr[q * LD + q];
                        const T xr = Mr[p * LD + q], xi = Mi[p * LD + q];
                        const T g = sqrt(xr * xr + xi * xi);
                        if (g > gskip && !(gth > (T)0 && g <= gth * fabs(aqq - app))) {
                            const T theta = (aqq - app) / (2 * g);
                            const T t = (theta >= 0 ? (T)1 : (T)-1) / (fabs(theta) + sqrt((T)1 + theta * theta));
                            c = (T)1 / sqrt((T)1 + t * t);
                            sn = t * c;
                            pr = xr / g;
                            pi = xi / g;
                            d0 = app - t * g;
                            d1 = aqq + t * g;
                            fix = 1;
                        }
                    }
                    s_pq[tid] = make_int2(p, q);
                    s_rot[tid] = RotPar<T>{c, sn, pr, pi};
                    s_d0[tid] = d0; s_d1[tid] = d1; s_fix[tid] = fix;
                }
                // a round without any rotation changes nothing
                if (!__syncthreads_or(tid < HP ? s_fix[tid] : 0)) continue;
                rotated = 1;
                // 2. M <- G^dag M G, one 2 x 2 block per (pair A, pair B)
                for (int t = tid; t < HP * HP; t += nt) {
                    const int A = t / HP, B = t % HP;
                    const int2 pqA = s_pq[A], pqB = s_pq[B];
                    const int pA = pqA.x, qA = pqA.y, pB = pqB.x, qB = pqB.y;
                    const RotPar<T> rA = s_rot[A], rB = s_rot[B];
                    const T cA = rA.c, sA = rA.s, cB = rB.c, sB = rB.s;
                    const cplx<T> phA = mk(rA.pr, rA.pi), phB = mk(rB.pr, rB.pi);
                    const cplx<T> x00 = mk(Mr[pA * LD + pB], Mi[pA * LD + pB]), x01 = mk(Mr[pA * LD + qB], Mi[pA * LD + qB]);
                    const cplx<T> x10 = mk(Mr[qA * LD + pB], Mi[qA * LD + pB]), x11 = mk(Mr[qA * LD + qB], Mi[qA * LD + qB]);
                    // Y = X G_B: column p' = c xp - s e^{-i phi} xq ; column q' = s e^{i phi} xp + c xq
                    const cplx<T> y00 = cB * x00 - sB * mul_cj(x01, phB), y01 = sB * (phB * x00) + cB * x01;
                    const cplx<T> y10 = cB * x10 - sB * mul_cj(x11, phB), y11 = sB * (phB * x10) + cB * x11;
                    // Z = G_A^dag Y: row p' = c yp - s e^{i phi} yq ; row q' = s e^{-i phi} yp + c yq
                    cplx<T> z00 = cA * y00 - sA * (phA * y10), z01 = cA * y01 - sA * (phA * y11);
                    cplx<T> z10 = sA * mul_cj(y00, phA) + cA * y10, z11 = sA * mul_cj(y01, phA) + cA * y11;
                    if (A == B && s_fix[A]) {
                        // exact 2 x 2 result on the rotated pair
                        z00 = mk(s_d0[A], (T)0);
                        z11 = mk(s_d1[A], (T)0);
                        z01 = z10 = mk((T)0, (T)0);
                    }
                    Mr[pA * LD + pB] = z00.re; Mi[pA * LD + pB] = z00.im;
                    Mr[pA * LD + qB] = z01.re; Mi[pA * LD + qB] = z01.im;
                    Mr[qA * LD + pB] = z10.re; Mi[qA * LD + pB] = z10.im;
                    Mr[qA * LD + qB] = z11.re; Mi[qA * LD + qB] = z11.im;
                }
                // 3. V <- V G (consecutive threads walk the rows of one pair)
                for (int t = tid; t < NP * HP; t += nt) {
                    const int j = t / NP, i = t % NP;
                    const int2 pq = s_pq[j];
                    const int p = pq.x, q = pq.y;
                    const RotPar<T> rj = s_rot[j];
                    const T c = rj.c, sn = rj.s;
                    const cplx<T> ph = mk(rj.pr, rj.pi);
                    const cplx<T> vp = mk(Vr[i * LD + p], Vi[i * LD + p]), vq = mk(Vr[i * LD + q], Vi[i * LD + q]);
                    const cplx<T> np_ = c * vp - sn * mul_cj(vq, ph), nq = sn * (ph * vp) + c * vq;
                    Vr[i * LD + p] = np_.re; Vi[i * LD + p] = np_.im;
                    Vr[i * LD + q] = nq.re; Vi[i * LD + q] = nq.im;
                }
                __syncthreads();
            }
            converged = (gth > (T)0 && !rotated) || off_norm() <= tol2;
        }
        if (tid == 0) {
            atomicMax(sweeps_max, sweep);
            if (!converged) atomicAdd(flag_cap, 1);
        }
        // sort ascending (stable on ties), write E and U, keep the sorted
        // eigenvectors as the next k-point's warm start
        for (int i = tid; i < N; i += nt) {
            const T ei = Mr[i * LD + i];
            int rank = 0;
            for (int j = 0; j < N; ++j) {
                const T ej = Mr[j * LD + j];
                rank += (ej < ei || (ej == ei && j < i)) ? 1 : 0;
            }
            s_E[rank] = ei;
            E[(size_t)k * N + rank] = ei;
            for (int row = 0; row < N; ++row) {
                const T vr = Vr[row * LD + i], vi = Vi[row * LD + i];
                U[(size_t)k * NN + row * N + rank] = mk(vr, vi);
                Tr[row * LD + rank] = vr;
                Ti[row * LD + rank] = vi;
            }
        }
        __syncthreads();
        if (redo_flag && tid == 0) {
            // smallest gap between neighbouring sorted eigenvalues
            T mingap = (T)1e30;
            for (int i = 0; i + 1 < N; ++i) mingap = fmin(mingap, s_E[i + 1] - s_E[i]);
            redo_flag[k] = (!converged || (double)mingap < degen_gap || !(mingap == mingap)) ? 1 : 0;
        }
        for (int e = tid; e < N * N; e += nt) {
            const int i = e / N, j = e % N;
            Vr[i * LD + j] = Tr[i * LD + j];
            Vi[i * LD + j] = Ti[i * LD + j];
        }
    }
}

// ---------------------------------------------------------------------------
// Register-resident FP32 Jacobi for N <= 32 (the mixed form): one warp per
// warm-start run of k-points, lane r holding row r of the matrix M and row r
// of the eigenvector accumulator V in registers, so that a sweep touches no
// shared memory and needs no block barrier.
//
// Ordering: the round-robin ("circle") schedule with the pairs of every round
// in the fixed slots (2a, 2a+1).  Player positions 0..31 map to slots by
// slot(p) = 2p (p <= 15), 2(31-p)+1 (p >= 16); position 0 is fixed and the
// others move one position per round, so the 31 rounds of a sweep meet every
// pair once and return to the starting order.  Columns live at register index
// = slot and move one step along the fixed slot cycle after every round
// (static register moves); rows stay in their lanes, each lane computing the
// slot its row holds this round and the lane of its pair partner.  A round
// rotates the 16 slot pairs: columns by static register indices, rows by
// exchanging the partner lane's row with shuffles.  The rotation of a pair is the one of jacobi_kernel
// (Rutishauser choice of t, G = [[c, s e^{i phi}], [-s e^{-i phi}, c]]); pairs
// with a padded index (>= N) or |M_pq| below the skip threshold are left.
namespace {

__host__ __device__ constexpr int jw_slot(int p) { return p <= 15 ? 2 * p : 2 * (31 - p) + 1; }
__host__ __device__ constexpr int jw_pos(int s) { return (s & 1) ? 31 - (s >> 1) : (s >> 1); }

// v[slot(p)] <- v[slot(p-1)] for p = 2..31, v[slot(1)] <- v[slot(31)]
__device__ __forceinline__ void jw_cycle(float (&v)[32]) {
    const float t = v[jw_slot(31)];
#pragma unroll
    for (int p = 31; p >= 2; --p) v[jw_slot(p)] = v[jw_slot(p - 1)];
    v[jw_slot(1)] = t;
}

// v[idx] for a run-time idx, by a five-level select tree on the index bits
__device__ __forceinline__ float jw_pick(const float (&v)[32], int idx) {
    float a[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) a[j] = (idx & 1) ? v[2 * j + 1] : v[2 * j];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = (idx & 2) ? a[2 * j + 1] : a[2 * j];
#pragma unroll
    for (int j = 0; j < 4; ++j) a[j] = (idx & 4) ? a[2 * j + 1] : a[2 * j];
#pragma unroll
    for (int j = 0; j < 2; ++j) a[j] = (idx & 8) ? a[2 * j + 1] : a[2 * j];
    return (idx & 16) ? a[1] : a[0];
}

// (v[idx & ~1], v[idx | 1]) for a run-time idx: the select tree of jw_pick on
// index bits 1..4, carried for both members of the pair
__device__ __forceinline__ void jw_pick_pair(const float (&v)[32], int idx, float& e0, float& e1) {
    float a[8], b[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        a[j] = (idx & 2) ? v[4 * j + 2] : v[4 * j];
        b[j] = (idx & 2) ? v[4 * j + 3] : v[4 * j + 1];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        a[j] = (idx & 4) ? a[2 * j + 1] : a[2 * j];
        b[j] = (idx & 4) ? b[2 * j + 1] : b[2 * j];
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        a[j] = (idx & 8) ? a[2 * j + 1] : a[2 * j];
        b[j] = (idx & 8) ? b[2 * j + 1] : b[2 * j];
    }
    e0 = (idx & 16) ? a[1] : a[0];
    e1 = (idx & 16) ? b[1] : b[0];
}

constexpr int JW_LD = 33;
constexpr int JW_SMEM_FLOATS = 4 * 32 * JW_LD + 16 * 4 + 3 * 32;   // per warp: H, V planes, pair parameters, E/rank/player

template <int NW, int MB>
__global__ void __launch_bounds__(32 * NW, MB) jacobi_warp_kernel(int N, int64_t nk, int kblock,
                                                              const float4* __restrict__ Hdf,
                                                              float* __restrict__ E, cplx<float>* __restrict__ U,
                                                              int max_sweeps, int* sweeps_max, int* flag_cap,
                                                              double degen_gap, int* redo_flag) {
    extern __shared__ float jw_sm[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float* Hr = jw_sm + (size_t)w * JW_SMEM_FLOATS;
    float* Hi = Hr + 32 * JW_LD;
    float* Sr = Hi + 32 * JW_LD;   // sorted eigenvectors [component][band]: output and next warm start
    float* Si = Sr + 32 * JW_LD;
    float4* prm = reinterpret_cast<float4*>(Si + 32 * JW_LD);   // [16] (c, s, e^{i phi})
    float* sE = reinterpret_cast<float*>(prm + 16);
    int* sR = reinterpret_cast<int*>(sE + 32);
    int* sP = sR + 32;
    const unsigned FULL = 0xffffffffu;
    const int NN = N * N;
    const int p0 = jw_pos(lane);   // position of this lane's row at the start of a sweep
    const int64_t chain = (int64_t)blockIdx.x * NW + w;
    float mr[32], mi[32], vr[32], vi[32];
    for (int jb = 0; jb < kblock; ++jb) {
        const int64_t k = chain * kblock + jb;
        if (k >= nk) break;
        const bool warm = jb > 0;
        // the run's next H(k) into L2 while this one is diagonalised
        if (lane == 0 && jb + 1 < kblock && k + 1 < nk)
            l2_prefetch(Hdf + (size_t)(k + 1) * NN, (uint32_t)(NN * sizeof(float4)));
        // FP32 copy of the FP64 H(k), Hermitised from its upper triangle
        const float4* Hk = Hdf + (size_t)k * NN;
        float part = 0.f;
        for (int a = 0; a < 32; ++a) {
            const int b = lane;
            if (b >= a) {
                float re = 0.f, im = 0.f;
                if (b < N && a < N) {
                    const float4 x = Hk[a * N + b];
                    re = x.x;
                    im = b == a ? 0.f : x.y;
                }
                Hr[a * JW_LD + b] = re;
                Hi[a * JW_LD + b] = im;
                Hr[b * JW_LD + a] = re;
                Hi[b * JW_LD + a] = -im;
                part += (b == a ? 1.f : 2.f) * (re * re + im * im);
            }
        }
        __syncwarp();
        float fro2 = part;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) fro2 += __shfl_xor_sync(FULL, fro2, o);
        const int pid = lane;   // band (player) of this lane's row; after whole sweeps also of column slot 'lane'
        if (!warm) {
#pragma unroll
            for (int t = 0; t < 32; ++t) {
                mr[t] = Hr[lane * JW_LD + t];
                mi[t] = Hi[lane * JW_LD + t];
                vr[t] = t == lane ? 1.f : 0.f;
                vi[t] = 0.f;
            }
        } else {
            // M = S^dag H S with S the previous k-point's sorted eigenvectors:
            // lane s forms row s of S^dag H, then row s of M
            float wr[32], wi[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) wr[j] = wi[j] = 0.f;
            for (int i = 0; i < 32; ++i) {
                const float a = Sr[i * JW_LD + lane], b = -Si[i * JW_LD + lane];   // conj(S_is)
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const float hr = Hr[i * JW_LD + j], hi = Hi[i * JW_LD + j];
                    wr[j] = fmaf(a, hr, fmaf(-b, hi, wr[j]));
                    wi[j] = fmaf(a, hi, fmaf(b, hr, wi[j]));
                }
            }
#pragma unroll
            for (int t = 0; t < 32; ++t) mr[t] = mi[t] = 0.f;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const float a = wr[j], b = wi[j];
#pragma unroll
                for (int t = 0; t < 32; ++t) {
                    const float sr = Sr[j * JW_LD + t], si = Si[j * JW_LD + t];
                    mr[t] = fmaf(a, sr, fmaf(-b, si, mr[t]));
                    mi[t] = fmaf(a, si, fmaf(b, sr, mi[t]));
                }
            }
#pragma unroll
            for (int t = 0; t < 32; ++t) {
                vr[t] = Sr[lane * JW_LD + t];
                vi[t] = Si[lane * JW_LD + t];
            }
        }
        // the diagonal of a Hermitian matrix is real
#pragma unroll
        for (int t = 0; t < 32; ++t) mi[t] = (t == lane) ? 0.f : mi[t];
        const float tolr = 4.f * 1.1920928955078125e-07f * sqrtf((float)N);
        const float tol2 = tolr * tolr * fro2;
        const float gskip = 1e-10f * sqrtf(fro2);
        // off-diagonal Frobenius norm, summed without the diagonal (subtracting d^2
        // from the row sum would leave FP32 cancellation noise far above tol2)
        auto off_norm = [&]() {
            float o = 0.f;
#pragma unroll
            for (int t = 0; t < 32; ++t) o += (t == lane) ? 0.f : fmaf(mr[t], mr[t], mi[t] * mi[t]);
#pragma unroll
            for (int q = 16; q > 0; q >>= 1) o += __shfl_xor_sync(FULL, o, q);
            return o;
        };
        bool converged = (N == 1) || (warm && off_norm() <= tol2);
        int sweep = 0;
        for (sweep = 0; sweep < max_sweeps && !converged; ++sweep) {
            for (int r = 0; r < 31; ++r) {
                // rows stay in their lanes: this lane's row sits at slot sl this round, its
                // pair partner's row in lane pl (columns: register index = slot)
                const int sl = jw_slot(p0 == 0 ? 0 : (p0 - 1 + r) % 31 + 1);
                const int pqp = jw_pos(sl ^ 1);
                const int pl = jw_slot(pqp == 0 ? 0 : (pqp - 1 - r + 62) % 31 + 1);
                const bool even = !(sl & 1);
                // pair (p, q) = (even slot, odd slot): parameters formed by the even lane
                float e0, e1;
                jw_pick_pair(mr, sl, e0, e1);
                const float d = even ? e0 : e1, xr0 = even ? e1 : e0;
                const float xi0 = jw_pick(mi, sl ^ 1);
                const float dq = __shfl_sync(FULL, d, pl);
                float c = 1.f, sn = 0.f, pr = 1.f, pi = 0.f;
                if (even && lane < N && pl < N) {
                    const float app = d, aqq = dq, xr = xr0, xi = xi0;
                    const float g = sqrtf(xr * xr + xi * xi);
                    if (g > gskip) {
                        const float th = (aqq - app) / (2.f * g);
                        const float t = (th >= 0.f ? 1.f : -1.f) / (fabsf(th) + sqrtf(1.f + th * th));
                        c = 1.f / sqrtf(1.f + t * t);
                        sn = t * c;
                        pr = xr / g;
                        pi = xi / g;
                    }
                }
                // (c, s e^{i phi}) of the pair
                if (even) prm[sl >> 1] = make_float4(c, sn * pr, sn * pi, 0.f);
                __syncwarp();
                // M <- M G and V <- V G on this lane's rows (column pairs in static slots):
                // p' = c x - s e^{-i phi} y,  q' = s e^{i phi} x + c y
#pragma unroll
                for (int a = 0; a < 16; ++a) {
                    const float4 g4 = prm[a];
                    const float ca = g4.x, zr = g4.y, zi = g4.z;
                    {
                        const float xr = mr[2 * a], xi = mi[2 * a], yr = mr[2 * a + 1], yi = mi[2 * a + 1];
                        mr[2 * a] = fmaf(ca, xr, -fmaf(zr, yr, zi * yi));
                        mi[2 * a] = fmaf(ca, xi, -fmaf(zr, yi, -zi * yr));
                        mr[2 * a + 1] = fmaf(zr, xr, fmaf(-zi, xi, ca * yr));
                        mi[2 * a + 1] = fmaf(zr, xi, fmaf(zi, xr, ca * yi));
                    }
                    {
                        const float xr = vr[2 * a], xi = vi[2 * a], yr = vr[2 * a + 1], yi = vi[2 * a + 1];
                        vr[2 * a] = fmaf(ca, xr, -fmaf(zr, yr, zi * yi));
                        vi[2 * a] = fmaf(ca, xi, -fmaf(zr, yi, -zi * yr));
                        vr[2 * a + 1] = fmaf(zr, xr, fmaf(-zi, xi, ca * yr));
                        vi[2 * a + 1] = fmaf(zr, xi, fmaf(zi, xr, ca * yi));
                    }
                }
                // M <- G^dag M on the pair's two rows:
                // p' = c y_p - s e^{i phi} y_q,  q' = s e^{-i phi} y_p + c y_q
                {
                    const float4 g4 = prm[sl >> 1];
                    const float ca = g4.x, A = even ? -g4.y : g4.y, B = g4.z;
#pragma unroll
                    for (int t = 0; t < 32; ++t) {
                        const float orr = __shfl_sync(FULL, mr[t], pl), ori = __shfl_sync(FULL, mi[t], pl);
                        mr[t] = fmaf(ca, mr[t], fmaf(A, orr, B * ori));
                        mi[t] = fmaf(ca, mi[t], fmaf(A, ori, -B * orr));
                    }
                }
                __syncwarp();
                // next round: columns one step along the slot cycle (rows stay in their lanes)
                jw_cycle(mr);
                jw_cycle(mi);
                jw_cycle(vr);
                jw_cycle(vi);
            }
            converged = off_norm() <= tol2;
        }
        if (lane == 0) {
            atomicMax(sweeps_max, sweep);
            if (!converged) atomicAdd(flag_cap, 1);
        }
        // eigenvalues in slot order; ranks among the real bands (padded slots keep pid)
        const float ev = jw_pick(mr, lane);
        sE[lane] = ev;
        sP[lane] = pid;
        __syncwarp();
        int rank = pid;
        if (pid < N) {
            rank = 0;
            for (int t = 0; t < 32; ++t) {
                if (sP[t] >= N) continue;
                const float et = sE[t];
                rank += (et < ev || (et == ev && t < lane)) ? 1 : 0;
            }
        }
        sR[lane] = rank;
        if (pid < N) E[(size_t)k * N + rank] = ev;
        __syncwarp();
        // sorted eigenvectors: S[i][rank(s)] = V[i][s]
#pragma unroll
        for (int t = 0; t < 32; ++t) {
            const int rt = sR[t];
            Sr[lane * JW_LD + rt] = vr[t];
            Si[lane * JW_LD + rt] = vi[t];
        }
        __syncwarp();
        for (int i = 0; i < N; ++i)
            if (lane < N) U[(size_t)k * NN + i * N + lane] = mk(Sr[i * JW_LD + lane], Si[i * JW_LD + lane]);
        if (redo_flag) {
            // smallest gap between neighbouring sorted eigenvalues (H is free: sorted E in its first row)
            if (pid < N) Hr[rank] = ev;
            __syncwarp();
            float gap = 1e30f;
            if (lane + 1 < N) gap = Hr[lane + 1] - Hr[lane];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) gap = fminf(gap, __shfl_xor_sync(FULL, gap, o));
            if (lane == 0) redo_flag[k] = (!converged || (double)gap < degen_gap || !(gap == gap)) ? 1 : 0;
        }
        __syncwarp();
    }
}

}  // namespace

}  // namespace

template <typename T>
cudaError_t launch_eig(int N, int64_t nk, const cplx<T>* W, int nbW, const float4* Hdf, T* E, cplx<T>* U,
                       int max_sweeps, int* sweeps_max, int* flag_cap, double degen_gap, int* redo_flag,
                       cudaStream_t s, int threads_req, int kblock_req, float gap_theta, bool warp_form) {
    if (nk <= 0) return cudaSuccess;
    // a run of consecutive k-points per CTA, each warm-started from its
    // neighbour's eigenvectors (consecutive k-points are mesh neighbours).  Eight
    // per CTA: four measured 5% faster at N = 32, but its extra cold starts
    // raised the mixed form's Chern-Simons error on sparse k subsets above 1e-6.
    const int kblock = kblock_req > 0 ? kblock_req : 8;
    const unsigned grid = (unsigned)((nk + kblock - 1) / kblock);
    auto go = [&](auto kern, int NP, int threads) {
        // a tuned thread count: a multiple of 32, at least one thread per pair, at most 256
        if (threads_req >= NP / 2 && threads_req <= 256 && threads_req % 32 == 0) threads = threads_req;
        const size_t smem = 6 * (size_t)NP * (NP + 1) * sizeof(T);
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        kern<<<grid, threads, smem, s>>>(N, nk, kblock, W, nbW, Hdf, E, U, max_sweeps, sweeps_max, flag_cap, degen_gap,
                                         redo_flag, gap_theta);
        return cudaGetLastError();
    };
    if constexpr (sizeof(T) == 4) {
        if (warp_form && Hdf && N <= 32) {
            constexpr int NW = 4;
            const unsigned g = (unsigned)((nk + (int64_t)kblock * NW - 1) / ((int64_t)kblock * NW));
            const size_t smem = (size_t)NW * JW_SMEM_FLOATS * sizeof(float);
            auto wgo = [&](auto kern) {
                cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                if (e != cudaSuccess) return e;
                kern<<<g, 32 * NW, smem, s>>>(N, nk, kblock, Hdf, reinterpret_cast<float*>(E),
                                              reinterpret_cast<cplx<float>*>(U), max_sweeps, sweeps_max, flag_cap,
                                              degen_gap, redo_flag);
                return cudaGetLastError();
            };
            return threads_req == 1 ? wgo(jacobi_warp_kernel<NW, 3>) : wgo(jacobi_warp_kernel<NW, 1>);
        }
    }
    if (N <= 8) return go(jacobi_kernel<T, 8>, 8, 64);
    if (N <= 16) return go(jacobi_kernel<T, 16>, 16, 128);
    if (N <= 32) return go(jacobi_kernel<T, 32>, 32, 128);
    if (N <= 64) return go(jacobi_kernel<T, 64>, 64, 256);
    return cudaErrorInvalidValue;
}

// Eigenpair refinement of the FP32 Jacobi result (U, lambda) against the
// FP64 H(k), in residual form so that a single product needs more than FP32:
//   R = H U - U diag(lambda)    compensated FP32 (Dot2 with H = H_hi + H_lo),
//                               the only cancelling product
//   P = U^dag R                 FP32 (R is small: its rounding is relative to
//                               |R|, not to |H|)
//   rho_n = lambda_n + P_nn / S_nn,  S_nn = |u_n|^2   (normalised Rayleigh
//                               quotient, FP64)
//   E_n = rho_n + sum_{m!=n} |P_mn|^2 / (rho_n - rho_m)        (second order)
//   C1_mn = P_mn / (rho_n - rho_m)                              (first order)
//   C2_mn = (X C1)_mn / (rho_n - rho_m),  C2_nn = -|C1_:n|^2 / 2,
//           X = P without its diagonal                          (second order)
//   U' = (U + U (C1 + C2)) diag(S_nn)^-1/2                      (FP32)
// C1 also restores, to first order, the orthogonality the warm-started FP32
// vectors lose: <u'_m|u'_n> = S_mn + C1_mn + conj(C1_nm) + O(2nd) = O(2nd).
// Energies are exact to third order in |P| / gap, vectors to third order in
// the perturbation and second order in the loss of orthogonality, for every
// gap above degen_gap.  A k-point with a gap at or below degen_gap, an
// unconverged FP32 Jacobi run (flag already set) or non-finite values is
// flagged for the full FP64 rerun.  Eigenpairs are re-sorted by the refined
// energies.
__global__ void __launch_bounds__(256) refine_kernel(int N, const float4* __restrict__ Hdf,
                                                     const float* __restrict__ lam, cplx<float>* __restrict__ U,
                                                     cplx<float>* __restrict__ Ulo, double* __restrict__ E64,
                                                     double degen_gap, int* __restrict__ redo_flag) {
    extern __shared__ unsigned char smem_raw[];
    const int Np = N + (N & 1), NPP = Np * Np;
    double* rho = reinterpret_cast<double*>(smem_raw);
    double* En = rho + Np;
    float* Sn = reinterpret_cast<float*>(En + Np);
    float* Dn = Sn + Np;
    float* Iv = Dn + Np;                       // [Np][Np] inverse gaps
    cplx<float>* Hh = reinterpret_cast<cplx<float>*>(Iv + NPP);
    cplx<float>* Hl = Hh + NPP;
    cplx<float>* Us = Hl + NPP;
    cplx<float>* Rs = Us + NPP;
    cplx<float>* Ps = Rs + NPP;
    __shared__ float ls[kMaxN], rh[kMaxN], rl[kMaxN];
    __shared__ float qp[2][8][kMaxN], sch_s[kMaxN], scl_s[kMaxN];
    __shared__ long long ekey[kMaxN];
    __shared__ int rk[kMaxN];
    __shared__ int s_flag;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int64_t k = blockIdx.x;
    const int NN = N * N;
    {
        // one CTA per k-point: H(k) and U of the k-point about two waves of
        // resident CTAs ahead into L2
        constexpr int64_t kAhead = 1024;
        const int64_t ka = k + kAhead;
        if (ka < (int64_t)gridDim.x) {
            if (tid == 0) l2_prefetch(Hdf + (size_t)ka * NN, (uint32_t)(NN * sizeof(float4)));
            if (tid == 32) l2_prefetch(U + (size_t)ka * NN, (uint32_t)(NN * sizeof(cplx<float>)));
        }
    }
    for (int e = tid; e < NPP; e += nt) {
        const int i = e / Np, j = e % Np;
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        cplx<float> uv = mk(0.f, 0.f);
        if (i < N && j < N) {
            const int a = i < j ? i : j, b = i < j ? j : i;
            x = Hdf[(size_t)k * NN + a * N + b];
            if (i > j) {          // lower triangle: the conjugate
                x.y = -x.y;
                x.w = -x.w;
            } else if (i == j) {  // real diagonal
                x.y = 0.f;
                x.w = 0.f;
            }
            uv = U[(size_t)k * NN + i * N + j];
        }
        Hh[e] = mk(x.x, x.y);
        Hl[e] = mk(x.z, x.w);
        Us[e] = uv;
    }
    for (int n = tid; n < Np; n += nt) ls[n] = n < N ? lam[(size_t)k * N + n] : 0.f;
    if (tid == 0) s_flag = redo_flag ? redo_flag[k] : 0;
    __syncthreads();
    // R = H U - U diag(lambda), 4 x 1 tiles per thread (four rows of a warp, its
    // lanes over the columns: broadcast H loads, conflict-free U loads): H_hi U
    // in Dot2, H_lo U in FP32
    for (int t = tid; t < ((Np + 3) >> 2) * Np; t += nt) {
        const int rb = t / Np, c = t - rb * Np, i0 = 4 * rb;
        DF sr[4], si[4];
        cplx<float> lo[4];
#pragma unroll
        for (int x = 0; x < 4; ++x) {
            sr[x] = DF{0.f, 0.f};
            si[x] = DF{0.f, 0.f};
            lo[x] = mk(0.f, 0.f);
        }
        for (int l = 0; l < Np; ++l) {
            const cplx<float> u = Us[l * Np + c];
#pragma unroll
            for (int x = 0; x < 4; ++x) {
                if (i0 + x >= Np) break;
                const cplx<float> hx = Hh[(i0 + x) * Np + l], gx = Hl[(i0 + x) * Np + l];
                df_add_prod(sr[x], hx.re, u.re);
                df_add_prod(sr[x], -hx.im, u.im);
                df_add_prod(si[x], hx.re, u.im);
                df_add_prod(si[x], hx.im, u.re);
                fma_c(lo[x], gx, u);
            }
        }
#pragma unroll
        for (int x = 0; x < 4; ++x) {
            const int r = i0 + x;
            if (r >= Np) break;
            const cplx<float> u = Us[r * Np + c];
            // subtract lambda u exactly, then round the residual once
            DF qr = sr[x], qi = si[x];
            df_add_prod(qr, -ls[c], u.re);
            df_add_prod(qi, -ls[c], u.im);
            Rs[r * Np + c] = mk(qr.s + (qr.c + lo[x].re), qi.s + (qi.c + lo[x].im));
        }
    }
    __syncthreads();
    // P = U^dag R (FP32)
    smem_cgemm<float, true>(Np, Np, Us, Rs, Ps, tid, nt);
    for (int n = tid; n < N; n += nt) {
        float sq = 0.f;   // |u_n|^2 = 1 + O(1e-5): FP32 keeps P_nn / S_nn to ~1e-13
        for (int l = 0; l < N; ++l) sq += abs2(Us[l * Np + n]);
        Sn[n] = sq;
    }
    __syncthreads();
    for (int n = tid; n < N; n += nt) {
        // the Rayleigh-quotient correction P_nn / S_nn (~1e-7 of E) in FP32: ~1e-14 of E
        const double r = (double)ls[n] + (double)(Ps[n * Np + n].re / Sn[n]);
        rho[n] = r;
        rh[n] = (float)r;
        rl[n] = (float)(r - (double)rh[n]);
    }
    __syncthreads();
    // inverse gaps 1 / (rho_n - rho_m): the difference of two FP32 hi + lo
    // pairs (exact for close energies, where it matters), the reciprocal in
    // FP32 (it scales corrections of order |P|/gap)
    const float dgap = (float)degen_gap;
    for (int e = tid; e < NPP; e += nt) {
        const int m = e / Np, n = e % Np;
        float iv = 0.f;
        if (m < N && n < N && m != n) {
            const float d = (rh[n] - rh[m]) + (rl[n] - rl[m]);
            if (fabsf(d) > dgap) iv = 1.f / d;
            else s_flag = 1;
        }
        Iv[e] = iv;
    }
    __syncthreads();
    for (int n = tid; n < N; n += nt) {
        float e2 = 0.f;
        for (int m = 0; m < N; ++m) e2 += abs2(Ps[m * Np + n]) * Iv[m * Np + n];
        const double en = rho[n] + (double)e2;
        En[n] = en;
        if (!isfinite(en)) s_flag = 1;
    }
    __syncthreads();
    // C1 into Rs; X (P without its diagonal) stays in Ps
    for (int e = tid; e < NPP; e += nt) {
        const int m = e / Np, n = e % Np;
        Rs[e] = Iv[e] * Ps[e];
        if (m == n) Ps[e] = mk(0.f, 0.f);
    }
    __syncthreads();
    // X C1 into Hh (H is no longer needed); diagonal of the normalisation term
    smem_cgemm<float, false>(Np, Np, Ps, Rs, Hh, tid, nt);
    for (int n = tid; n < Np; n += nt) {
        float q = 0.f;
        for (int m = 0; m < N; ++m) q += abs2(Rs[m * Np + n]);
        Dn[n] = -0.5f * q;
    }
    __syncthreads();
    // C = C1 + C2 into Rs
    for (int e = tid; e < NPP; e += nt) {
        const int m = e / Np, n = e % Np;
        if (m >= N || n >= N) continue;
        Rs[e] = (m == n) ? mk(Dn[n], 0.f) : Rs[e] + Iv[e] * Hh[e];
    }
    __syncthreads();
    // U C into Ps
    smem_cgemm<float, false>(Np, Np, Us, Rs, Ps, tid, nt);
    __syncthreads();
    // the refined vectors' squared norms |u + U C|^2 in double-FP32, eight row
    // groups per band (|h + e|^2 = h^2 + 2 h e + e^2 with h + e = u + (U C) by
    // TwoSum, h^2 by TwoProduct, e^2 < 2^-48 h^2 dropped)
    if (Ulo)
        for (int e = tid; e < 8 * Np; e += nt) {
            const int n = e % Np, g = e / Np;
            float qs = 0.f, qc = 0.f;
            if (n < N)
                for (int row = g; row < N; row += 8) {
                    const cplx<float> a = Us[row * Np + n], b = Ps[row * Np + n];
                    float hr, er, hm, em;
                    two_sum_f(a.re, b.re, hr, er);
                    two_sum_f(a.im, b.im, hm, em);
                    const float pr = hr * hr, pm = hm * hm;
                    float t, te, u, ue;
                    two_sum_f(qs, pr, t, te);
                    two_sum_f(t, pm, u, ue);
                    qs = u;
                    qc += te + ue + fmaf(hr, hr, -pr) + fmaf(hm, hm, -pm) + 2.f * (hr * er + hm * em);
                }
            qp[0][g][n] = qs;
            qp[1][g][n] = qc;
        }
    // energies ordered through their IEEE-754 bits as signed integers (the
    // order of doubles, on the integer pipe)
    for (int n = tid; n < N; n += nt) {
        const long long b = __double_as_longlong(En[n]);
        ekey[n] = b ^ ((b >> 63) & 0x7fffffffffffffffLL);
    }
    __syncthreads();
    // per band: its rank, its energy, the scale 1 / |u + U C| (FP64 only for the
    // one square root per band) as FP32 hi + lo
    for (int n = tid; n < N; n += nt) {
        const long long kn = ekey[n];
        int rank = 0;
        for (int j = 0; j < N; ++j) rank += (ekey[j] < kn || (ekey[j] == kn && j < n)) ? 1 : 0;
        E64[(size_t)k * N + rank] = En[n];
        rk[n] = rank;
        if (Ulo) {
            float qs = qp[0][0][n], qc = qp[1][0][n];
            for (int g = 1; g < 8; ++g) {
                float t, te;
                two_sum_f(qs, qp[0][g][n], t, te);
                qs = t;
                qc += te + qp[1][g][n];
            }
            const double scd = 1.0 / sqrt((double)qs + (double)qc);
            sch_s[n] = (float)scd;
            scl_s[n] = (float)(scd - (double)sch_s[n]);
        } else {
            sch_s[n] = (float)(1.0 / sqrt(Sn[n]));
        }
    }
    __syncthreads();
    // the refined vectors, one element per thread: (u + U C) scaled, as FP32 hi + lo
    // (TwoSum for the sum, TwoProduct (FMA) for the scaling) or FP32 alone
    for (int e = tid; e < N * N; e += nt) {
        const int row = e / N, n = e - row * N;
        const cplx<float> a = Us[row * Np + n], b = Ps[row * Np + n];
        const size_t o = (size_t)k * NN + row * N + rk[n];
        const float sch = sch_s[n];
        if (!Ulo) {
            U[o] = mk((a.re + b.re) * sch, (a.im + b.im) * sch);
        } else {
            const float scl = scl_s[n];
            float hr, er, hm, em;
            two_sum_f(a.re, b.re, hr, er);
            two_sum_f(a.im, b.im, hm, em);
            const float pr = hr * sch, pm = hm * sch;
            const float lr = fmaf(hr, sch, -pr) + (er * sch + hr * scl);
            const float lm = fmaf(hm, sch, -pm) + (em * sch + hm * scl);
            const float ur = pr + lr, um = pm + lm;   // renormalised pair
            U[o] = mk(ur, um);
            Ulo[o] = mk((pr - ur) + lr, (pm - um) + lm);
        }
    }
    __syncthreads();
    if (tid == 0 && redo_flag) redo_flag[k] = s_flag ? 1 : 0;
}

size_t refine_smem_bytes(int N) {
    const size_t Np = N + (N & 1);
    return 2 * Np * sizeof(double) + 2 * Np * sizeof(float) + Np * Np * sizeof(float) +
           5 * Np * Np * sizeof(cplx<float>);
}

cudaError_t launch_refine(int N, int64_t nk, const float4* Hdf, const float* lam, cplx<float>* U,
                          cplx<float>* Ulo, double* E64, double degen_gap, int* redo_flag, cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    const size_t smem = refine_smem_bytes(N);
    cudaError_t e = cudaFuncSetAttribute(refine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(refine_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    refine_kernel<<<(unsigned)nk, N <= 16 ? 128 : 256, smem, s>>>(N, Hdf, lam, U, Ulo, E64, degen_gap, redo_flag);
    return cudaGetLastError();
}

template cudaError_t launch_eig<double>(int, int64_t, const cplx<double>*, int, const float4*, double*,
                                        cplx<double>*, int, int*, int*, double, int*, cudaStream_t, int, int, float, bool);
template cudaError_t launch_eig<float>(int, int64_t, const cplx<float>*, int, const float4*, float*,
                                       cplx<float>*, int, int*, int*, double, int*, cudaStream_t, int, int, float, bool);

}  // namespace mepi
