// W -> Hbar gauge rotation of rotate_gauge (src/wann_interp.f90:502-550) on
// the tensor cores, for the mixed form with n_wf <= 32:
//     Hbar_a = U^dag H_a U,  Abar_a = U^dag A_a U   (a = x,y,z; D1 position)
// and the band diagonal of U^dag Omega_q U (the only part of the curvature the
// band sums consume, src/mep_niu.f90:35, src/kubo_mep.f90:35).
//
// Arithmetic: exact-slice ("Ozaki") products on FP16 tensor cores.  Every
// operand row is scaled by a power of two 2^e >= its largest magnitude and
// written as four balanced base-512 digits,
//     x = 2^(e-8) (d1 + d2/512 + d3/512^2 + d4/512^3),  |d_p| <= 256,
// each digit an integer that FP16 holds exactly.  A digit product d_p e_q is
// an integer of magnitude at most 2^16 and a K = 64 sum of them at most 2^22,
// so the FP32 tensor-memory accumulator sums the (at most four) (p,q) pairs of
// one level L = p + q exactly (|sum| <= 2^24).  For the tile of the velocity
// blocks levels 2..5 are kept (10 digit GEMMs): at K = 64 the product is
// typically within 2^-32 of the product of its row and column scales (2^-28 in
// the worst case of extreme digits with aligned signs), below the FP32
// rounding of the inputs, which matches the compensated (Dot2) CUDA-core
// rotation it replaces.  The connection and curvature tiles use three digits
// and levels 2..4 (6 digit GEMMs; typically 2^-23, at worst 2^-19), the
// accuracy of the plain FP32 rotation those blocks had on the CUDA cores.
// The levels are combined in double-FP32 (TwoSum).  The refined eigenvectors
// enter as FP32 hi + lo pairs, so U carries about 35 bits into the products.
//
// Complex products as real GEMMs, K = 64 (real parts, then imaginary parts):
//   GEMM1  [T_r | T_i] = [X_r | X_i] . [[U_r, U_i], [-U_i, U_r]]   (T = X U)
//   GEMM2  [Y_r | Y_i] = [T_r^T | -T_i^T] . (the same U operand)    (Y = T^dag U)
// so both GEMMs share the U digits (operand B, N = 64).  Operand A stacks four
// 32-row blocks (M = 128): GEMM1 tiles hold (H_x, H_y, H_z, A_x),
// (A_y, A_z, Om_1, Om_2) and (Om_3); GEMM2 tiles the rotated blocks of the
// first two.  The transpose T -> T^dag happens as the GEMM1 accumulator is read:
// TMEM lane n of warp quarter q holds row n of T_q, and its digits are stored
// into column n of the GEMM2 operand rows.  The Hermitian W-gauge blocks are
// read from their upper triangle by columns (coalesced) and turned into rows by
// a warp-shuffle transpose.  The curvature diagonal
// d_n = sum_i conj(U_in) T_in is a cross-lane sum of the GEMM1 rows.
//
// One CTA (8 warps; warp w reads TMEM lanes 32 (w % 4).. and the real
// (w < 4) or imaginary (w >= 4) column half) walks k-points with stride
// gridDim.x, two CTAs per SM so that one's digit work overlaps the other's
// MMAs.  Operands are K-major with the 128-byte swizzle the MMA descriptor
// expects; one thread issues the tcgen05.mma and commits to an mbarrier whose
// waits are bounded: on a timeout the CTA raises *err, waits (bounded) for its
// MMAs in flight, frees its tensor memory and returns.
#include <cuda_fp16.h>

#include <algorithm>

#include "mepi_internal.cuh"
#include "tc_common.cuh"

namespace mepi {

namespace {

using namespace tc;

constexpr int RT_THREADS = 256;
constexpr int RT_NP = 32;                           // padded band count
constexpr uint32_t RT_A_DIG = 128 * 128;            // 128 rows x 64 FP16 (one digit of operand A)
constexpr uint32_t RT_B_DIG = 64 * 128;             // 64 rows x 64 FP16 (one digit of operand B)
constexpr uint32_t RT_TMEM_COLS = 256;              // 4 levels x 64 FP32 columns
// kind::f16, FP32 accumulator, FP16 A and B, both K-major, N = 64, M = 128
constexpr uint32_t RT_IDESC = (1u << 4) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
constexpr int RT_LD = RT_NP + 1;                    // row stride of the U planes

struct RtSmem {
    // (dynamic shared memory, 1024-byte aligned) A digits, B digits, then:
    float ur[RT_NP * RT_LD], ui[RT_NP * RT_LD];     // U planes (hi parts), U[i][n]
    int a_exp[128];                                 // GEMM2 operand A row exponents
    int b_exp[64];                                  // operand B row exponents
    float fsc[32];                                  // 2^(f_j - 16) per output column j
    float c2[4][32];                                // 2^(8 - e2) per GEMM2 operand row (q, m)
    float half_max[2][128];                         // row (or column) maxima of the two halves
    float omr[2][4][32], omi[2][4][32];             // curvature diagonals, per column half
    uint64_t bar;
    uint32_t tmem;
    int abort;
};
constexpr size_t RT_SMEM = 4 * RT_A_DIG + 4 * RT_B_DIG + sizeof(RtSmem) + 1024;

// exponent e with |x| < 2^e for a positive x, held to [-60, 64] (a row below
// 2^-60 is represented against 2^-60, i.e. as zero digits); 0 for zero
__device__ __forceinline__ int exp_above(float x) {
    const int b = (__float_as_int(x) >> 23) & 0xff;
    return b == 0 ? 0 : min(max(b - 126, -60), 64);
}
// 2^e, the exponent held to the normal range
__device__ __forceinline__ float pow2f(int e) {
    return __int_as_float((min(max(e, -126), 127) + 127) << 23);
}

// byte offset of element (row, k) in a 128-byte-swizzled K-major tile of FP16
__device__ __forceinline__ uint32_t sw_off(int row, int k) {
    return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((((k >> 3) ^ row) & 7) << 4) + (k & 7) * 2);
}

// four balanced base-512 digits of y (|y| <= 256, y given as hi + lo)
__device__ __forceinline__ void digits4(float hi, float lo, float (&d)[4]) {
    d[0] = rintf(hi);
    float r = ((hi - d[0]) + lo) * 512.f;
    d[1] = rintf(r);
    r = (r - d[1]) * 512.f;
    d[2] = rintf(r);
    r = (r - d[2]) * 512.f;
    d[3] = rintf(r);
}

// write 8 consecutive K elements (one 16-byte chunk) of the first nd digits
// of already scaled hi + lo values
__device__ __forceinline__ void store_chunk(unsigned char* tile0, uint32_t dig_bytes, int row, int chunk,
                                            const float (&vh)[8], const float (&vl)[8], int nd = 4) {
    float d[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i) digits4(vh[i], vl[i], d[i]);
    const uint32_t off = (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + (((chunk ^ row) & 7) << 4));
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        if (p >= nd) break;
        __half2 h0 = __floats2half2_rn(d[0][p], d[1][p]), h1 = __floats2half2_rn(d[2][p], d[3][p]);
        __half2 h2 = __floats2half2_rn(d[4][p], d[5][p]), h3 = __floats2half2_rn(d[6][p], d[7][p]);
        uint4 u;
        u.x = *reinterpret_cast<uint32_t*>(&h0);
        u.y = *reinterpret_cast<uint32_t*>(&h1);
        u.z = *reinterpret_cast<uint32_t*>(&h2);
        u.w = *reinterpret_cast<uint32_t*>(&h3);
        *reinterpret_cast<uint4*>(tile0 + p * dig_bytes + off) = u;
    }
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// level accumulators P2..P5 of one column -> hi + lo of P2 + P3/512 + P4/512^2 + P5/512^3
__device__ __forceinline__ void combine(float p2, float p3, float p4, float p5, float& hi, float& lo) {
    float e;
    two_sum(p2, p3 * (1.f / 512.f), hi, e);
    lo = e + fmaf(p4, 1.f / 262144.f, p5 * (1.f / 134217728.f));
}

// 32 values per lane -> lane l holds the max (or sum) over the warp of entry l
template <bool kMax>
__device__ __forceinline__ float transpose_reduce(float (&v)[32], int lane) {
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const bool up = (lane & s) != 0;
#pragma unroll
        for (int i = 0; i < s; ++i) {
            const float send = up ? v[i] : v[i + s];
            const float keep = up ? v[i + s] : v[i];
            const float recv = __shfl_xor_sync(0xffffffffu, send, s);
            v[i] = kMax ? fmaxf(keep, recv) : keep + recv;
        }
    }
    return v[0];
}

// 32 x 32 transpose across the warp: lane l holds column l (v[r] = M(r, l))
// on entry and row l (v[c] = M(l, c)) on exit -- five butterfly stages that
// swap one index bit with one lane bit, all register indices static
__device__ __forceinline__ void transpose32(float (&v)[32], int lane) {
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const bool b = (lane & s) != 0;
#pragma unroll
        for (int a = 0; a < 32; ++a) {
            if (a & s) continue;
            const float send = b ? v[a] : v[a + s];
            const float recv = __shfl_xor_sync(0xffffffffu, send, s);
            v[a] = b ? recv : v[a];
            v[a + s] = b ? v[a + s] : recv;
        }
    }
}

// 8 columns of the level accumulators (levels 2..nd+1) -> hi + lo per column
__device__ __forceinline__ void load_levels8(uint32_t taddr, float (&hi)[8], float (&lo)[8], int nd = 4) {
    float p2[8], p3[8], p4[8], p5[8];
    tmem_ld8(taddr, p2);
    tmem_ld8(taddr + 64, p3);
    tmem_ld8(taddr + 128, p4);
    if (nd == 4) {
        tmem_ld8(taddr + 192, p5);
    } else {
#pragma unroll
        for (int i = 0; i < 8; ++i) p5[i] = 0.f;
    }
    tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 8; ++i) combine(p2[i], p3[i], p4[i], p5[i], hi[i], lo[i]);
}

// the digit GEMMs of one tile: levels L = p + q = 2..nd+1 (p, q <= nd) into
// columns 64 (L-2): ten GEMMs with four digits, six with three
__device__ __forceinline__ void issue_tile(uint32_t tmem, const unsigned char* A, const unsigned char* B, uint64_t* bar,
                                           int nd) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
    for (int L = 2; L <= 5; ++L) {
        if (L > nd + 1) break;
        bool first = true;
#pragma unroll
        for (int p = 1; p <= 4; ++p) {
            const int q = L - p;
            if (p > nd || q < 1 || q > nd) continue;
            const uint64_t ad = sw128_desc(A + (p - 1) * RT_A_DIG), bd = sw128_desc(B + (q - 1) * RT_B_DIG);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                mma_f16(tmem + (uint32_t)(64 * (L - 2)), ad + 2 * kk, bd + 2 * kk, RT_IDESC, first ? 0u : 1u);
                first = false;
            }
        }
    }
    mma_commit(bar);
}

__global__ void __launch_bounds__(RT_THREADS, 2)
    rot_tc_kernel(int N, int nbW, int nrot, int nomega, int64_t nk, const cplx<float>* __restrict__ W,
                  const cplx<float>* __restrict__ Ug, const cplx<float>* __restrict__ Ulo,
                  cplx<float>* __restrict__ HA, cplx<float>* __restrict__ OD, int* err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    unsigned char* Adig = smem;
    unsigned char* Bdig = smem + 4 * RT_A_DIG;
    RtSmem& S = *reinterpret_cast<RtSmem*>(Bdig + 4 * RT_B_DIG);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int q = warp & 3, h = warp >> 2;   // TMEM lane quarter (block of the tile), column half
    const int NN = N * N;
    const FastDiv byN(N), byNN(NN);
    const int nblk = nrot + nomega;          // W blocks 1..nblk are rotated
    const int ntile = (nblk + 3) / 4;

    if (tid == 0) {
        mbar_init(&S.bar, 1);
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                     "r"(RT_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = S.tmem;
    const uint32_t tlane = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * h);   // my lanes, my column half
    uint32_t phase = 0;
    int issued = 0;
    // digits per operand in the current tile: four for the tile of the velocity
    // blocks (H_x, H_y, H_z, A_x: typically 2^-32 of the scales), three for the
    // connection and curvature tiles (typically 2^-23, the FP32 level these
    // blocks need: six digit GEMMs instead of ten, three levels to read back)
    int nd = 4;

    // digit stores -> async proxy, then one thread issues the tile's MMAs
    auto launch_mma = [&]() {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            issue_tile(tmem, Adig, Bdig, &S.bar, nd);
            ++issued;
        }
    };
    // bounded wait for the MMAs; the decision to go on is uniform over the CTA
    auto wait_mma = [&]() -> bool {
        if (!mbar_wait(&S.bar, phase)) S.abort = 1;
        __syncthreads();
        if (S.abort) return false;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        return true;
    };

    bool ok = true;
    for (int64_t k = blockIdx.x; k < nk && ok; k += gridDim.x) {
        // the next k-point of this CTA into L2 while this one is worked on: its W
        // blocks (one prefetch per block) and eigenvectors
        const int64_t kn = k + gridDim.x;
        if (tid < nblk + 2 && kn < nk) {
            const uint32_t bb = (uint32_t)(NN * sizeof(cplx<float>));
            if (tid < nblk)
                l2_prefetch(W + ((size_t)kn * nbW + 1 + tid) * NN, bb);
            else if (tid == nblk)
                l2_prefetch(Ug + (size_t)kn * NN, bb);
            else if (Ulo)
                l2_prefetch(Ulo + (size_t)kn * NN, bb);
        }
        __syncthreads();
        // ---- U planes (hi parts, for the curvature diagonal and the B exponents) ----
        const cplx<float>* Uk = Ug + (size_t)k * NN;
        for (int e = tid; e < RT_NP * RT_NP; e += RT_THREADS) {
            const int i = e >> 5, n = e & 31;
            const cplx<float> u = (i < N && n < N) ? Uk[i * N + n] : mk(0.f, 0.f);
            S.ur[i * RT_LD + n] = u.re;
            S.ui[i * RT_LD + n] = u.im;
        }
        __syncthreads();
        if (tid < 32) {   // B rows j and 32 + j hold column j of U: one exponent
            float mx = 0.f;
            for (int i = 0; i < RT_NP; ++i)
                mx = fmaxf(mx, fmaxf(fabsf(S.ur[i * RT_LD + tid]), fabsf(S.ui[i * RT_LD + tid])));
            const int e = exp_above(mx);
            S.b_exp[tid] = e;
            S.b_exp[tid + 32] = e;
            S.fsc[tid] = pow2f(e - 16);
        }
        __syncthreads();
        {
            // thread -> B row j (0..63), K quarter (16 elements = 2 chunks); the
            // refined eigenvectors enter as hi + lo (FP32 pairs), read from global
            const int j = tid >> 2, kq = tid & 3;
            const int col = j & 31;
            const float sc = pow2f(8 - S.b_exp[j]);
            const cplx<float>* Ulk = Ulo ? Ulo + (size_t)k * NN : nullptr;
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const int chunk = 2 * kq + cc;      // K = 8 chunk .. 8 chunk + 7
                float vh[8], vl[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const int kx = 8 * chunk + t, i = kx & 31;
                    const bool in = i < N && col < N;
                    const cplx<float> uh = in ? Uk[i * N + col] : mk(0.f, 0.f);
                    const cplx<float> ul = (in && Ulk) ? Ulk[i * N + col] : mk(0.f, 0.f);
                    // row j < 32: (U_r[:, j] | -U_i[:, j]);  row 32 + j: (U_i[:, j] | U_r[:, j])
                    const bool take_re = (j < 32) == (kx < 32);
                    const float sg = (j < 32 && kx >= 32) ? -1.f : 1.f;
                    vh[t] = sg * (take_re ? uh.re : uh.im) * sc;
                    vl[t] = sg * (take_re ? ul.re : ul.im) * sc;
                }
                store_chunk(Bdig, RT_B_DIG, j, chunk, vh, vl);
            }
        }

        for (int tile = 0; tile < ntile; ++tile) {
            nd = tile == 0 ? 4 : 3;
            // ---- GEMM1 operand A: rows (q, n) = [X_r(n,:) | X_i(n,:)] of W block 1 + 4 tile + q ----
            const int blk = 4 * tile + q;            // 0-based rotated block (W block blk + 1)
            const bool present = blk < nblk;
            const bool rot = present && blk < nrot;
            const bool omega = present && blk >= nrot;
            const int nrot_tile = max(0, min(4, nrot - 4 * tile));   // rotated blocks in this tile
            const int n = lane, row = 32 * q + lane;
            float xv[32];
            float mx = 0.f;
#pragma unroll
            for (int m = 0; m < 32; ++m) xv[m] = 0.f;
            if (present) {
                // only the component this warp needs, Re (h = 0) or Im (h = 1).  The
                // block's upper triangle U' (diagonal halved for Re, zero for Im) is
                // read by columns, lane n holding U'(m, n) for every m (one coalesced
                // load per m), and transposed across the warp to the rows U'(n, m);
                // row n of the Hermitian block is then X_r = U'_r + U'_r^T,
                // X_i = U'_i - U'_i^T.
                const float* Wf = reinterpret_cast<const float*>(W + ((size_t)k * nbW + 1 + blk) * NN) + h;
                float tv[32];
#pragma unroll
                for (int m = 0; m < 32; ++m) {
                    float v = 0.f;
                    if (m <= n && n < N) v = Wf[2 * (m * N + n)];
                    if (m == n) v = h == 0 ? 0.5f * v : 0.f;
                    xv[m] = v;
                    tv[m] = v;
                }
                transpose32(tv, lane);
#pragma unroll
                for (int m = 0; m < 32; ++m) {
                    xv[m] = h == 0 ? xv[m] + tv[m] : tv[m] - xv[m];
                    mx = fmaxf(mx, fabsf(xv[m]));
                }
            }
            S.half_max[h][row] = mx;
            __syncthreads();
            const int ea = exp_above(fmaxf(S.half_max[0][row], S.half_max[1][row]));
            {
                const float sc = pow2f(8 - ea);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float vh[8], vl[8];
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        vh[t] = xv[8 * c + t] * sc;
                        vl[t] = 0.f;
                    }
                    store_chunk(Adig, RT_A_DIG, row, 4 * h + c, vh, vl, nd);
                }
            }
            launch_mma();
            if (!(ok = wait_mma())) break;
            const float pa = pow2f(ea);

            // ---- GEMM1 accumulator, row n of T_q: T(n, j) = 2^(ea + f_j - 16) (hi + lo) ----
            // pass 1: column maxima (rotated blocks) or the curvature diagonal (Omega blocks)
            float acc[32], acc2[32];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float hi[8], lo[8];
                load_levels8(tlane + 8 * c, hi, lo, nd);
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int j = 8 * c + i;
                    const float t = hi[i] * (pa * S.fsc[j]);
                    if (omega) {
                        // d_j = sum_i conj(U_ij) T_ij (lane n is row i = n):
                        // h = 0 (t = Re T): Re += ur t, Im -= ui t;  h = 1 (t = Im T): Re += ui t, Im += ur t
                        const float ur = S.ur[n * RT_LD + j], ui = S.ui[n * RT_LD + j];
                        acc[j] = h == 0 ? ur * t : ui * t;
                        acc2[j] = h == 0 ? -ui * t : ur * t;
                    } else {
                        acc[j] = rot ? fabsf(t) : 0.f;
                        acc2[j] = 0.f;
                    }
                }
            }
            if (omega) {
                const float sr = transpose_reduce<false>(acc, lane);
                const float si = transpose_reduce<false>(acc2, lane);
                S.omr[h][q][lane] = sr;
                S.omi[h][q][lane] = si;
            }
            const float cmax = omega ? 0.f : transpose_reduce<true>(acc, lane);   // column j = lane of T_q
            __syncthreads();   // every thread has read the row maxima: reuse half_max for the column maxima
            S.half_max[h][row] = cmax;
            __syncthreads();
            if (h == 0) {   // GEMM2 operand row (q, m = lane): exponent and digit scale
                const int e2 = exp_above(fmaxf(S.half_max[0][row], S.half_max[1][row]));
                S.a_exp[row] = e2;
                S.c2[q][lane] = pow2f(8 - e2);
            }
            __syncthreads();
            if (omega && h == 0 && lane < N)
                OD[((size_t)k * nomega + (blk - nrot)) * N + lane] =
                    mk(S.omr[0][q][lane] + S.omr[1][q][lane], S.omi[0][q][lane] + S.omi[1][q][lane]);
            if (nrot_tile == 0) continue;
            // pass 2: GEMM2 operand A rows (q, m) = [T_r(:, m) | -T_i(:, m)]; lane n -> K = n + 32 h.
            // Rows of quarters without a rotated block keep stale digits; their output is not read.
            if (rot) {
                const int kx = n + 32 * h;
#pragma unroll 1
                for (int c = 0; c < 4; ++c) {
                    float hi[8], lo[8];
                    load_levels8(tlane + 8 * c, hi, lo, nd);
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int j = 8 * c + i;
                        const float sc = pa * S.fsc[j] * S.c2[q][j] * (h == 0 ? 1.f : -1.f);
                        float d[4];
                        digits4(hi[i] * sc, lo[i] * sc, d);
                        const uint32_t off = sw_off(32 * q + j, kx);
#pragma unroll
                        for (int p = 0; p < 4; ++p)
                            if (p < nd) *reinterpret_cast<__half*>(Adig + p * RT_A_DIG + off) = __float2half_rn(d[p]);
                    }
                }
            }
            launch_mma();
            if (!(ok = wait_mma())) break;
            // ---- GEMM2 accumulator, lane m: Y_q(m, j) = 2^(e2_m + f_j - 16) (hi + lo) ----
            // staged as real and imaginary planes [128 rows][33] (conflict-free row writes)
            float* stage = reinterpret_cast<float*>(Adig);
            if (rot) {
                const float pe2 = pow2f(S.a_exp[row]);
                float* pl = stage + h * (128 * RT_LD) + row * RT_LD;
#pragma unroll 1
                for (int c = 0; c < 4; ++c) {
                    float hi[8], lo[8];
                    load_levels8(tlane + 8 * c, hi, lo, nd);
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int j = 8 * c + i;
                        pl[j] = (hi[i] + lo[i]) * (pe2 * S.fsc[j]);
                    }
                }
            }
            __syncthreads();
            // coalesced copy of the rotated blocks of this tile to HA[k][blk][m][j], Hermitian
            // by construction: the strictly lower triangle mirrors the upper one and the
            // diagonal is real, so that the gauge commutators cancel as exactly as their terms
            for (int e = tid; e < nrot_tile * NN; e += RT_THREADS) {
                const int bq = byNN.div(e), r = e - bq * NN, m = byN.div(r), j = r - m * N;
                const int o = (32 * bq + (m <= j ? m : j)) * RT_LD + (m <= j ? j : m);
                const float vr = stage[o], vi = stage[128 * RT_LD + o];
                HA[((size_t)k * 6 + 4 * tile + bq) * NN + r] = mk(vr, m < j ? vi : (m > j ? -vi : 0.f));
            }
        }
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    // on an abort, let the MMAs in flight finish before tensor memory is freed
    __syncthreads();
    if (tid == 0 && !ok && issued > 0) mbar_wait(&S.bar, phase);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(RT_TMEM_COLS) : "memory");
    }
}

}  // namespace

bool rot_tc_supported(const DevModel& m) { return m.do_gauge && m.N <= RT_NP && m.N >= 1; }

cudaError_t launch_rot_tc(const DevModel& m, int64_t nk, const cplx<float>* W, const cplx<float>* U,
                          const cplx<float>* Ulo, cplx<float>* HA, cplx<float>* OD, int* err, cudaStream_t s) {
    if (nk <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(rot_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RT_SMEM);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const int64_t grid = std::min<int64_t>(nk, 2 * (int64_t)sms);
    const int nrot = m.has_r ? 6 : 3, nomega = m.has_r ? 3 : 0;
    rot_tc_kernel<<<(unsigned)grid, RT_THREADS, RT_SMEM, s>>>(m.N, m.nb, nrot, nomega, nk, W, U, Ulo, HA, OD, err);
    return cudaGetLastError();
}

}  // namespace mepi
