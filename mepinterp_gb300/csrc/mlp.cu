// Proposal network of the adaptive k-mesh refinement (include/mepi_mlp.h).
//
// A fully connected network n_in -> 128 x depth (GELU) -> 1.  Every layer
// product is a BF16 GEMM on the tensor cores, C[m][n] = sum_k A[m][k] B[n][k]
// with A and B K-contiguous, staged by TMA into a 4-stage shared-memory ring
// with a 128-byte swizzle, issued by one thread as tcgen05.mma kind::f16 with
// BF16 operands and an FP32 accumulator in tensor memory, and read back by
// four epilogue warps with tcgen05.ld (the pipeline of the tensor-core
// Fourier GEMM, ft_tc.cu).  Per layer l with input H_{l-1} (rows = samples):
//   forward          Z_l = H_{l-1} W_l^T + b_l,  H_l = bf16(gelu(Z_l))
//   backward, data   dH_{l-1} = dZ_l W_l           (B operand: W_l^T, kept in BF16)
//   backward, weight dW_l = dZ_l^T H_{l-1}         (K = samples, split over CTAs,
//                                                   partials summed in a fixed order)
// The elementwise kernels (bias + GELU, GELU', the head, the reductions and
// Adam) run in FP32; activations and their gradients are rounded to BF16
// where they become GEMM operands, and are written in both orientations so
// that every GEMM reads K-contiguous operands.  One training step is captured
// into a CUDA graph; the batch index and Adam step live in device memory so
// that the graph replays unchanged.  Results are deterministic: no atomics
// touch the sums.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/mepi.h"
#include "../../include/mepi_mlp.h"
#include "tc_common.cuh"

namespace mepi {
namespace {

using namespace tc;
typedef __nv_bfloat16 bf16;

constexpr int kWidth = 128;
constexpr int kInPad = 64;        // input features padded to one 128-byte K block
constexpr int kMaxDepth = 8;
constexpr int kMaxRows = 32768;   // rows per device pass
constexpr int GBM = 128, GBK = 64, GSTAGES = 4, GTHREADS = 192;
constexpr int kRowsPerSplit = 128;  // samples (K) per CTA of a weight-gradient GEMM
constexpr int kEwRows = 32;         // rows per CTA of the elementwise kernels
constexpr int kHeadRows = 8;        // rows per CTA of the head (one warp each)

// ---------------------------------------------------------------------------
// BF16 GEMM
template <int BN>
__global__ void __launch_bounds__(GTHREADS, 1)
    gemm_bf16_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int nkb,
                     float* __restrict__ C, int ldc, size_t split_stride, int* err) {
    constexpr uint32_t A_BYTES = GBM * GBK * 2;
    constexpr uint32_t B_BYTES = BN * GBK * 2;
    constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
    constexpr uint32_t TMEM_COLS = BN;
    // kind::f16 descriptor: FP32 accumulator, A and B both BF16, K-major, N = BN, M = 128
    constexpr uint32_t IDESC =
        (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(GBM >> 4) << 24);

    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + GSTAGES * STAGE_BYTES);
    uint64_t* empty = full + GSTAGES;
    uint64_t* accum = empty + GSTAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_tile = blockIdx.x, m_tile = blockIdx.y;
    const int kb0 = blockIdx.z * nkb;
    C += (size_t)blockIdx.z * split_stride;

    if (threadIdx.x == 0) {
        for (int s = 0; s < GSTAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    int issued = 0;
    if (warp == 0 && lane == 0) {
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % GSTAGES;
            const uint32_t ph = (uint32_t)(kb / GSTAGES) & 1u;
            if (*abort_flag) break;
            if (!mbar_wait(&empty[s], ph ^ 1u)) {
                *abort_flag = 1;
                atomicExch(err, 1);
                break;
            }
            unsigned char* st = smem + s * STAGE_BYTES;
            mbar_expect_tx(&full[s], STAGE_BYTES);
            tma_load_2d(st, &tmA, (kb0 + kb) * GBK, m_tile * GBM, &full[s]);
            tma_load_2d(st + A_BYTES, &tmB, (kb0 + kb) * GBK, n_tile * BN, &full[s]);
            ++issued;
        }
    } else if (warp == 1 && lane == 0) {
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % GSTAGES;
            const uint32_t ph = (uint32_t)(kb / GSTAGES) & 1u;
            if (*abort_flag || !mbar_wait(&full[s], ph)) {
                *abort_flag = 1;
                atomicExch(err, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            unsigned char* st = smem + s * STAGE_BYTES;
            const uint64_t ad = sw128_desc(st), bd = sw128_desc(st + A_BYTES);
#pragma unroll
            for (int kk = 0; kk < GBK / 16; ++kk) {
                const uint64_t off = (uint64_t)(kk * 32) >> 4;   // 16 BF16 = 32 bytes along K
                mma_f16(tmem, ad + off, bd + off, IDESC, (kb | kk) != 0 ? 1u : 0u);
            }
            mma_commit(&empty[s]);
        }
        mma_commit(accum);
    } else if (warp >= 2) {
        const bool ok = mbar_wait(accum, 0);
        if (!ok) {
            *abort_flag = 1;
            atomicExch(err, 1);
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int quad = warp & 3;
        const int row = m_tile * GBM + quad * 32 + lane;
        const uint32_t tbase = tmem + ((uint32_t)(quad * 32) << 16);
        float* Crow = C + (size_t)row * ldc + (size_t)n_tile * BN;
        for (int c8 = 0; c8 < BN / 8; ++c8) {
            float v[8];
            tmem_ld8(tbase + (uint32_t)(8 * c8), v);
            tmem_wait_ld();
            if (!ok) continue;
            reinterpret_cast<float4*>(Crow + 8 * c8)[0] = make_float4(v[0], v[1], v[2], v[3]);
            reinterpret_cast<float4*>(Crow + 8 * c8)[1] = make_float4(v[4], v[5], v[6], v[7]);
        }
    }
    __syncwarp();
    if (warp == 0 && lane == 0 && *abort_flag) {
        for (int kb = issued - GSTAGES > 0 ? issued - GSTAGES : 0; kb < issued; ++kb)
            mbar_wait(&full[kb % GSTAGES], (uint32_t)(kb / GSTAGES) & 1u);
    }
    if (warp == 1 && lane == 0 && *abort_flag) mbar_wait(accum, 0);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

template <int BN>
constexpr size_t gemm_smem() {
    return (size_t)GSTAGES * (GBM * GBK * 2 + BN * GBK * 2) + 1024 + 256;
}

// ---------------------------------------------------------------------------
// elementwise kernels
__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z) {
    // d/dz [z Phi(z)] = Phi(z) + z phi(z)
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// Gather the batch rows: row r of the batch is sample order[base + r] (order
// null: sample r when r < n_valid); -1 marks a padding row.  base =
// (*step) * rows.
__global__ void pack_kernel(const float* __restrict__ x, int n_in, const float* __restrict__ y,
                            const int* __restrict__ order, const int* __restrict__ step, int rows, int n_valid,
                            int ld_t, bf16* __restrict__ X0, bf16* __restrict__ X0t, float* __restrict__ yb,
                            float* __restrict__ mask) {
    const int c = threadIdx.x;   // input column, 0..63
    const int64_t base = order ? (int64_t)(*step) * rows : 0;
    for (int rr = 0; rr < kEwRows; ++rr) {
        const int r = blockIdx.x * kEwRows + rr;
        const int src = order ? order[base + r] : (r < n_valid ? r : -1);
        const float v = (src >= 0 && c < n_in) ? x[(size_t)src * n_in + c] : 0.f;
        const bf16 b = __float2bfloat16_rn(v);
        X0[(size_t)r * kInPad + c] = b;
        X0t[(size_t)c * ld_t + r] = b;
        if (c == 0) {
            yb[r] = (src >= 0 && y) ? y[src] : 0.f;
            mask[r] = src >= 0 ? 1.f : 0.f;
        }
    }
}

// Z = C + b, H = bf16(gelu(Z)) (and its transpose); Z and Ht may be null (inference)
__global__ void bias_gelu_kernel(const float* __restrict__ C, const float* __restrict__ b, float* __restrict__ Z,
                                 bf16* __restrict__ H, bf16* __restrict__ Ht, int ld_t) {
    const int o = threadIdx.x;
    const float bo = b[o];
    for (int rr = 0; rr < kEwRows; ++rr) {
        const int r = blockIdx.x * kEwRows + rr;
        const float z = C[(size_t)r * kWidth + o] + bo;
        const bf16 h = __float2bfloat16_rn(gelu(z));
        if (Z) Z[(size_t)r * kWidth + o] = z;
        H[(size_t)r * kWidth + o] = h;
        if (Ht) Ht[(size_t)o * ld_t + r] = h;
    }
}

// Head f = H . w_o + b_o, one warp per row.  Training (dH non-null): squared
// error against yb over the masked rows scaled by inv_count[*step],
// dH = dout w_o, and per-CTA partials of grad w_o, grad b_o and the loss.
__global__ void head_kernel(const bf16* __restrict__ H, const float* __restrict__ wo, const float* __restrict__ bo,
                            const float* __restrict__ yb, const float* __restrict__ mask,
                            const float* __restrict__ inv_count, const int* __restrict__ step, float* __restrict__ out,
                            float* __restrict__ dH, float* __restrict__ part_wo, float* __restrict__ part_scalar) {
    __shared__ float sh[kHeadRows][kWidth];
    __shared__ float sd[kHeadRows][2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * kHeadRows + warp;
    float h[4], s = 0.f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        h[j] = __bfloat162float(H[(size_t)r * kWidth + lane + 32 * j]);
        s = fmaf(h[j], wo[lane + 32 * j], s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const float f = s + bo[0];
    if (out && lane == 0) out[r] = f;
    if (!dH) return;
    const float ic = inv_count[step ? *step : 0];
    const float e = (f - yb[r]) * mask[r];
    const float dout = 2.f * e * ic;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        dH[(size_t)r * kWidth + lane + 32 * j] = dout * wo[lane + 32 * j];
        sh[warp][lane + 32 * j] = dout * h[j];
    }
    if (lane == 0) {
        sd[warp][0] = dout;
        sd[warp][1] = e * e * ic;
    }
    __syncthreads();
    if (threadIdx.x < kWidth) {
        float a = 0.f;
        for (int w = 0; w < kHeadRows; ++w) a += sh[w][threadIdx.x];
        part_wo[(size_t)blockIdx.x * kWidth + threadIdx.x] = a;
    } else if (threadIdx.x < kWidth + 2) {
        const int q = threadIdx.x - kWidth;
        float a = 0.f;
        for (int w = 0; w < kHeadRows; ++w) a += sd[w][q];
        part_scalar[(size_t)blockIdx.x * 2 + q] = a;
    }
}

// dZ = dH * gelu'(Z) in FP32, stored as BF16 in both orientations; per-CTA
// partial of the bias gradient (from the FP32 values)
__global__ void gelu_back_kernel(const float* __restrict__ dH, const float* __restrict__ Z, bf16* __restrict__ dZ,
                                 bf16* __restrict__ dZt, int ld_t, float* __restrict__ part_b) {
    const int o = threadIdx.x;
    float acc = 0.f;
    for (int rr = 0; rr < kEwRows; ++rr) {
        const int r = blockIdx.x * kEwRows + rr;
        const float g = dH[(size_t)r * kWidth + o] * gelu_d(Z[(size_t)r * kWidth + o]);
        const bf16 b = __float2bfloat16_rn(g);
        dZ[(size_t)r * kWidth + o] = b;
        dZt[(size_t)o * ld_t + r] = b;
        acc += g;
    }
    part_b[(size_t)blockIdx.x * kWidth + o] = acc;
}

// out[i] = sum_p part[p * stride + src(i)] in p order; src(i) maps a dense
// (rows x cols_out) index to (row, col) of a (rows x cols_in) slice.
__global__ void sum_parts_kernel(const float* __restrict__ part, int n_parts, size_t stride, int rows, int cols_in,
                                 int cols_out, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols_out) return;
    const size_t src = (size_t)(i / cols_out) * cols_in + (i % cols_out);
    float a = 0.f;
    for (int p = 0; p < n_parts; ++p) a += part[(size_t)p * stride + src];
    out[i] = a;
}

// grad b_o and the loss of this step (into loss_hist[*step] when given)
__global__ void head_scalars_kernel(const float* __restrict__ part_scalar, int n_parts, float* __restrict__ g_bo,
                                    const int* __restrict__ step, float* __restrict__ loss_hist, double* loss_out) {
    if (threadIdx.x != 0) return;
    double a = 0.0, l = 0.0;
    for (int p = 0; p < n_parts; ++p) {
        a += part_scalar[2 * p];
        l += part_scalar[2 * p + 1];
    }
    *g_bo = (float)a;
    if (loss_hist) loss_hist[step ? *step : 0] = (float)l;
    if (loss_out) *loss_out = l;
}

struct NetDev {
    int depth, n_in;
    int in[kMaxDepth];
    int64_t offW[kMaxDepth], offb[kMaxDepth], off_wo, off_bo;
    bf16* Wb[kMaxDepth];   // W_l, (128 x in_pad) row-major, in_pad = 64 for l = 0
    bf16* Wt[kMaxDepth];   // W_l^T (in x 128), l >= 1
};

__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, int64_t n, float lr, const int* __restrict__ step) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float t = (float)(*step + 1);
    const float mi = b1 * m[i] + (1.f - b1) * g[i];
    const float vi = b2 * v[i] + (1.f - b2) * g[i] * g[i];
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.f - powf(b1, t)), vh = vi / (1.f - powf(b2, t));
    p[i] -= lr * mh / (sqrtf(vh) + eps);
}

// BF16 copies of the layer weights (row-major and transposed); the last
// thread advances the step counter.
__global__ void cast_weights_kernel(NetDev nd, const float* __restrict__ p, int* step) {
    const int l = blockIdx.y;
    if (l >= nd.depth) return;
    const int in_l = nd.in[l], in_pad = l == 0 ? kInPad : kWidth;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kWidth * in_pad; e += gridDim.x * blockDim.x) {
        const int o = e / in_pad, i = e % in_pad;
        const float w = i < in_l ? p[nd.offW[l] + (int64_t)o * in_l + i] : 0.f;
        const bf16 b = __float2bfloat16_rn(w);
        nd.Wb[l][e] = b;
        if (l > 0) nd.Wt[l][(size_t)i * kWidth + o] = b;
    }
    if (step && l == 0 && blockIdx.x == 0 && threadIdx.x == 0) *step += 1;
}

// ---------------------------------------------------------------------------
struct Arena {
    char* base = nullptr;
    size_t used = 0, cap = 0;
    template <typename X> X* take(size_t n) {
        X* r = reinterpret_cast<X*>(base + used);
        used += (n * sizeof(X) + 255) & ~(size_t)255;
        return r;
    }
};

}  // namespace
}  // namespace mepi

using namespace mepi;

struct mepi_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    NetDev nd{};
    int64_t n_params = 0;
    float *p = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;   // FP32 master, Adam moments, gradient
    int* step = nullptr;       // device Adam step / batch counter
    int* err = nullptr;        // device flag: a bounded wait in a GEMM timed out
    bf16* wbuf = nullptr;      // BF16 weight copies
    // row buffers for `cap` rows
    int cap = 0;
    void* arena = nullptr;
    bf16 *X0 = nullptr, *X0t = nullptr;
    float *yb = nullptr, *mask = nullptr, *Cb = nullptr, *dH = nullptr, *out = nullptr;
    float* Z[kMaxDepth] = {};
    bf16 *H[kMaxDepth] = {}, *Ht[kMaxDepth] = {}, *dZ[kMaxDepth] = {}, *dZt[kMaxDepth] = {};
    float *Wpart = nullptr, *part_b = nullptr, *part_wo = nullptr, *part_s = nullptr, *inv_one = nullptr;
    double* loss_d = nullptr;
    CUtensorMap tmX0, tmX0t, tmW[kMaxDepth], tmWt[kMaxDepth], tmH[kMaxDepth], tmHt[kMaxDepth], tmdZ[kMaxDepth],
        tmdZt[kMaxDepth];
};

namespace {

int free_rows(mepi_mlp* n) {
    if (n->arena) cudaFree(n->arena);
    n->arena = nullptr;
    n->cap = 0;
    return MEPI_OK;
}

// row buffers and their tensor maps for `rows` rows (a multiple of 128)
int ensure_rows(mepi_mlp* n, int rows) {
    if (rows <= n->cap) return MEPI_OK;
    free_rows(n);
    const int L = n->nd.depth;
    const size_t R = (size_t)rows;
    size_t bytes = 0;
    auto add = [&](size_t b) { bytes += (b + 255) & ~(size_t)255; };
    add(R * kInPad * 2); add(R * kInPad * 2); add(R * 4); add(R * 4); add(R * kWidth * 4); add(R * kWidth * 4);
    add(R * 4);
    for (int l = 0; l < L; ++l) {
        add(R * kWidth * 4);
        for (int q = 0; q < 4; ++q) add(R * kWidth * 2);
    }
    add((R / kRowsPerSplit) * kWidth * kWidth * 4);
    add((R / kEwRows) * kWidth * 4);
    add((R / kHeadRows) * kWidth * 4);
    add((R / kHeadRows) * 2 * 4);
    add(4);
    add(8);
    if (cudaMalloc(&n->arena, bytes) != cudaSuccess) {
        n->arena = nullptr;
        return MEPI_ERR_NOMEM;
    }
    Arena a{static_cast<char*>(n->arena), 0, bytes};
    n->X0 = a.take<bf16>(R * kInPad);
    n->X0t = a.take<bf16>(R * kInPad);
    n->yb = a.take<float>(R);
    n->mask = a.take<float>(R);
    n->Cb = a.take<float>(R * kWidth);
    n->dH = a.take<float>(R * kWidth);
    n->out = a.take<float>(R);
    for (int l = 0; l < L; ++l) {
        n->Z[l] = a.take<float>(R * kWidth);
        n->H[l] = a.take<bf16>(R * kWidth);
        n->Ht[l] = a.take<bf16>(R * kWidth);
        n->dZ[l] = a.take<bf16>(R * kWidth);
        n->dZt[l] = a.take<bf16>(R * kWidth);
    }
    n->Wpart = a.take<float>((R / kRowsPerSplit) * kWidth * kWidth);
    n->part_b = a.take<float>((R / kEwRows) * kWidth);
    n->part_wo = a.take<float>((R / kHeadRows) * kWidth);
    n->part_s = a.take<float>((R / kHeadRows) * 2);
    n->inv_one = a.take<float>(1);
    n->loss_d = a.take<double>(1);
    const CUtensorMapDataType BF = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    bool ok = encode_2d(&n->tmX0, n->X0, kInPad, R, GBK, GBM, BF) &&
              encode_2d(&n->tmX0t, n->X0t, R, kInPad, GBK, kInPad, BF);
    for (int l = 0; l < L && ok; ++l)
        ok = encode_2d(&n->tmH[l], n->H[l], kWidth, R, GBK, GBM, BF) &&
             encode_2d(&n->tmHt[l], n->Ht[l], R, kWidth, GBK, kWidth, BF) &&
             encode_2d(&n->tmdZ[l], n->dZ[l], kWidth, R, GBK, GBM, BF) &&
             encode_2d(&n->tmdZt[l], n->dZt[l], R, kWidth, GBK, kWidth, BF);
    if (!ok) {
        free_rows(n);
        return MEPI_ERR_CUDA;
    }
    n->cap = rows;
    return MEPI_OK;
}

template <int BN>
cudaError_t gemm(const CUtensorMap& A, const CUtensorMap& B, int M, int N, int K, int splits, float* C, int ldc,
                 int* err, cudaStream_t s) {
    const dim3 grid((unsigned)(N / BN), (unsigned)(M / GBM), (unsigned)splits);
    gemm_bf16_kernel<BN><<<grid, GTHREADS, gemm_smem<BN>(), s>>>(A, B, K / GBK / splits, C, ldc,
                                                                (size_t)M * ldc, err);
    return cudaGetLastError();
}

#define MLP_CK(x)                                  \
    do {                                           \
        if ((x) != cudaSuccess) return MEPI_ERR_CUDA; \
    } while (0)

// forward through every layer for `rows` rows already packed; training keeps Z and H^T
int enqueue_forward(mepi_mlp* n, int rows, bool train) {
    const int L = n->nd.depth;
    const int ld_t = n->cap;
    for (int l = 0; l < L; ++l) {
        const CUtensorMap& A = l == 0 ? n->tmX0 : n->tmH[l - 1];
        MLP_CK(gemm<128>(A, n->tmW[l], rows, kWidth, l == 0 ? kInPad : kWidth, 1, n->Cb, kWidth, n->err, n->stream));
        bias_gelu_kernel<<<rows / kEwRows, kWidth, 0, n->stream>>>(n->Cb, n->p + n->nd.offb[l], train ? n->Z[l] : nullptr,
                                                                   n->H[l], train ? n->Ht[l] : nullptr, ld_t);
        MLP_CK(cudaGetLastError());
    }
    return MEPI_OK;
}

// loss and gradient of a packed batch of `rows` rows into n->g
int enqueue_backward(mepi_mlp* n, int rows, const float* inv_count, const int* step, float* loss_hist,
                     double* loss_out) {
    const int L = n->nd.depth;
    const int ld_t = n->cap;
    const NetDev& nd = n->nd;
    head_kernel<<<rows / kHeadRows, kHeadRows * 32, 0, n->stream>>>(n->H[L - 1], n->p + nd.off_wo, n->p + nd.off_bo,
                                                                     n->yb, n->mask, inv_count, step, nullptr, n->dH,
                                                                     n->part_wo, n->part_s);
    MLP_CK(cudaGetLastError());
    sum_parts_kernel<<<1, kWidth, 0, n->stream>>>(n->part_wo, rows / kHeadRows, kWidth, 1, kWidth, kWidth,
                                                  n->g + nd.off_wo);
    head_scalars_kernel<<<1, 32, 0, n->stream>>>(n->part_s, rows / kHeadRows, n->g + nd.off_bo, step, loss_hist,
                                                 loss_out);
    MLP_CK(cudaGetLastError());
    for (int l = L - 1; l >= 0; --l) {
        gelu_back_kernel<<<rows / kEwRows, kWidth, 0, n->stream>>>(n->dH, n->Z[l], n->dZ[l], n->dZt[l], ld_t,
                                                                   n->part_b);
        sum_parts_kernel<<<1, kWidth, 0, n->stream>>>(n->part_b, rows / kEwRows, kWidth, 1, kWidth, kWidth,
                                                      n->g + nd.offb[l]);
        MLP_CK(cudaGetLastError());
        const int splits = rows / kRowsPerSplit;
        if (l == 0) {
            MLP_CK(gemm<64>(n->tmdZt[0], n->tmX0t, kWidth, kInPad, rows, splits, n->Wpart, kInPad, n->err, n->stream));
            const int tot = kWidth * nd.in[0];
            sum_parts_kernel<<<(tot + 255) / 256, 256, 0, n->stream>>>(n->Wpart, splits, (size_t)kWidth * kInPad,
                                                                       kWidth, kInPad, nd.in[0], n->g + nd.offW[0]);
        } else {
            MLP_CK(gemm<128>(n->tmdZt[l], n->tmHt[l - 1], kWidth, kWidth, rows, splits, n->Wpart, kWidth, n->err,
                             n->stream));
            sum_parts_kernel<<<kWidth * kWidth / 256, 256, 0, n->stream>>>(n->Wpart, splits, (size_t)kWidth * kWidth,
                                                                         kWidth, kWidth, kWidth, n->g + nd.offW[l]);
            // dH_{l-1} = dZ_l W_l
            MLP_CK(gemm<128>(n->tmdZ[l], n->tmWt[l], rows, kWidth, kWidth, 1, n->dH, kWidth, n->err, n->stream));
        }
        MLP_CK(cudaGetLastError());
    }
    return MEPI_OK;
}

int refresh_weights(mepi_mlp* n, int* step) {
    cast_weights_kernel<<<dim3(32, n->nd.depth), 256, 0, n->stream>>>(n->nd, n->p, step);
    MLP_CK(cudaGetLastError());
    return MEPI_OK;
}

int check_err(mepi_mlp* n) {
    MLP_CK(cudaStreamSynchronize(n->stream));
    int e = 0;
    MLP_CK(cudaMemcpy(&e, n->err, sizeof(int), cudaMemcpyDeviceToHost));
    return e ? MEPI_ERR_CUDA : MEPI_OK;
}

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return ((splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

int round_rows(int64_t r) { return (int)(((r + GBM - 1) / GBM) * GBM); }

}  // namespace

extern "C" {

int mepi_mlp_create(mepi_mlp** out, int32_t n_in, int32_t width, int32_t depth, uint64_t seed) {
    if (!out) return MEPI_ERR_ARG;
    *out = nullptr;
    if (n_in < 1 || n_in > kInPad || width != kWidth || depth < 1 || depth > kMaxDepth) return MEPI_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return MEPI_ERR_CUDA;
    }
    mepi_mlp* n = new (std::nothrow) mepi_mlp();
    if (!n) return MEPI_ERR_NOMEM;
    cudaGetDevice(&n->device);
    NetDev& nd = n->nd;
    nd.depth = depth;
    nd.n_in = n_in;
    int64_t off = 0;
    for (int l = 0; l < depth; ++l) {
        nd.in[l] = l == 0 ? n_in : kWidth;
        nd.offW[l] = off;
        off += (int64_t)kWidth * nd.in[l];
        nd.offb[l] = off;
        off += kWidth;
    }
    nd.off_wo = off;
    off += kWidth;
    nd.off_bo = off;
    off += 1;
    n->n_params = off;
    std::vector<float> h(off, 0.f);
    uint64_t st = seed;
    for (int l = 0; l < depth; ++l) {
        const double sd = 1.0 / std::sqrt((double)nd.in[l]);
        for (int64_t i = 0; i < (int64_t)kWidth * nd.in[l]; ++i) {
            const double u1 = uniform01(st), u2 = uniform01(st);
            h[nd.offW[l] + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
    for (int i = 0; i < kWidth; ++i) {
        const double u1 = uniform01(st), u2 = uniform01(st);
        h[nd.off_wo + i] =
            (float)(std::sqrt(1.0 / kWidth) * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
    }
    auto fail = [&](int rc) {
        mepi_mlp_destroy(n);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(MEPI_ERR_CUDA);
    if (cudaMalloc(&n->p, 4 * off * sizeof(float)) != cudaSuccess) return fail(MEPI_ERR_NOMEM);
    n->m = n->p + off;
    n->v = n->m + off;
    n->g = n->v + off;
    if (cudaMalloc(&n->step, 2 * sizeof(int)) != cudaSuccess) return fail(MEPI_ERR_NOMEM);
    n->err = n->step + 1;
    size_t wel = (size_t)kWidth * kInPad + (size_t)(depth - 1) * 2 * kWidth * kWidth;
    if (cudaMalloc(&n->wbuf, wel * sizeof(bf16)) != cudaSuccess) return fail(MEPI_ERR_NOMEM);
    bf16* w = n->wbuf;
    nd.Wb[0] = w;
    nd.Wt[0] = nullptr;
    w += (size_t)kWidth * kInPad;
    for (int l = 1; l < depth; ++l) {
        nd.Wb[l] = w;
        nd.Wt[l] = w + (size_t)kWidth * kWidth;
        w += 2 * (size_t)kWidth * kWidth;
    }
    const CUtensorMapDataType BF = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    if (!encode_2d(&n->tmW[0], nd.Wb[0], kInPad, kWidth, GBK, GBM, BF)) return fail(MEPI_ERR_CUDA);
    for (int l = 1; l < depth; ++l)
        if (!encode_2d(&n->tmW[l], nd.Wb[l], kWidth, kWidth, GBK, GBM, BF) ||
            !encode_2d(&n->tmWt[l], nd.Wt[l], kWidth, kWidth, GBK, GBM, BF))
            return fail(MEPI_ERR_CUDA);
    if (cudaFuncSetAttribute(gemm_bf16_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gemm_smem<128>()) != cudaSuccess ||
        cudaFuncSetAttribute(gemm_bf16_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gemm_smem<64>()) != cudaSuccess)
        return fail(MEPI_ERR_CUDA);
    *out = n;
    const int rc = mepi_mlp_set_params(n, h.data());
    if (rc) {
        *out = nullptr;
        return fail(rc);
    }
    return MEPI_OK;
}

int mepi_mlp_destroy(mepi_mlp* n) {
    if (!n) return MEPI_OK;
    cudaSetDevice(n->device);
    if (n->stream) cudaStreamSynchronize(n->stream);
    free_rows(n);
    for (void* q : {(void*)n->p, (void*)n->step, (void*)n->wbuf})
        if (q) cudaFree(q);
    if (n->stream) cudaStreamDestroy(n->stream);
    delete n;
    return MEPI_OK;
}

int64_t mepi_mlp_param_count(const mepi_mlp* n) { return n ? n->n_params : -1; }

int mepi_mlp_get_params(const mepi_mlp* n, float* params) {
    if (!n || !params) return MEPI_ERR_ARG;
    if (cudaSetDevice(n->device) != cudaSuccess) return MEPI_ERR_CUDA;
    MLP_CK(cudaStreamSynchronize(n->stream));
    MLP_CK(cudaMemcpy(params, n->p, n->n_params * sizeof(float), cudaMemcpyDeviceToHost));
    return MEPI_OK;
}

int mepi_mlp_set_params(mepi_mlp* n, const float* params) {
    if (!n || !params) return MEPI_ERR_ARG;
    for (int64_t i = 0; i < n->n_params; ++i)
        if (!std::isfinite(params[i])) return MEPI_ERR_ARG;
    if (cudaSetDevice(n->device) != cudaSuccess) return MEPI_ERR_CUDA;
    MLP_CK(cudaMemcpyAsync(n->p, params, n->n_params * sizeof(float), cudaMemcpyHostToDevice, n->stream));
    MLP_CK(cudaMemsetAsync(n->m, 0, 2 * n->n_params * sizeof(float), n->stream));
    MLP_CK(cudaMemsetAsync(n->step, 0, 2 * sizeof(int), n->stream));
    if (int rc = refresh_weights(n, nullptr)) return rc;
    MLP_CK(cudaStreamSynchronize(n->stream));
    return MEPI_OK;
}

int mepi_mlp_forward(mepi_mlp* n, int64_t n_rows, const float* x, float* y) {
    if (!n || n_rows < 0 || (n_rows > 0 && (!x || !y))) return MEPI_ERR_ARG;
    if (n_rows == 0) return MEPI_OK;
    if (cudaSetDevice(n->device) != cudaSuccess) return MEPI_ERR_CUDA;
    const int rows_max = (int)std::min<int64_t>(round_rows(n_rows), kMaxRows);
    if (int rc = ensure_rows(n, rows_max)) return rc;
    const int n_in = n->nd.n_in;
    float* dx = nullptr;
    MLP_CK(cudaMalloc(&dx, (size_t)rows_max * n_in * sizeof(float)));
    int rc = MEPI_OK;
    for (int64_t r0 = 0; r0 < n_rows && !rc; r0 += rows_max) {
        const int nv = (int)std::min<int64_t>(rows_max, n_rows - r0);
        const int rows = round_rows(nv);
        if (cudaMemcpyAsync(dx, x + r0 * n_in, (size_t)nv * n_in * sizeof(float), cudaMemcpyHostToDevice,
                            n->stream) != cudaSuccess) {
            rc = MEPI_ERR_CUDA;
            break;
        }
        pack_kernel<<<rows / kEwRows, kInPad, 0, n->stream>>>(dx, n_in, nullptr, nullptr, nullptr, rows, nv, n->cap,
                                                             n->X0, n->X0t, n->yb, n->mask);
        rc = enqueue_forward(n, rows, false);
        if (rc) break;
        const int L = n->nd.depth;
        head_kernel<<<rows / kHeadRows, kHeadRows * 32, 0, n->stream>>>(n->H[L - 1], n->p + n->nd.off_wo,
                                                                         n->p + n->nd.off_bo, nullptr, nullptr, nullptr,
                                                                         nullptr, n->out, nullptr, nullptr, nullptr);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(y + r0, n->out, (size_t)nv * sizeof(float), cudaMemcpyDeviceToHost, n->stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(n->stream) != cudaSuccess)
            rc = MEPI_ERR_CUDA;
    }
    cudaFree(dx);
    if (!rc) rc = check_err(n);
    return rc;
}

int mepi_mlp_loss_grad(mepi_mlp* n, int64_t n_rows, const float* x, const float* y, double* loss, float* grad) {
    if (!n || n_rows < 1 || n_rows > kMaxRows || !x || !y) return MEPI_ERR_ARG;
    if (cudaSetDevice(n->device) != cudaSuccess) return MEPI_ERR_CUDA;
    const int rows = round_rows(n_rows);
    if (int rc = ensure_rows(n, rows)) return rc;
    const int n_in = n->nd.n_in;
    float* dx = nullptr;
    MLP_CK(cudaMalloc(&dx, (size_t)n_rows * (n_in + 1) * sizeof(float)));
    float* dy = dx + (size_t)n_rows * n_in;
    const float ic = 1.f / (float)n_rows;
    int rc = MEPI_OK;
    if (cudaMemcpyAsync(dx, x, (size_t)n_rows * n_in * sizeof(float), cudaMemcpyHostToDevice, n->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(dy, y, (size_t)n_rows * sizeof(float), cudaMemcpyHostToDevice, n->stream) != cudaSuccess ||
        cudaMemcpyAsync(n->inv_one, &ic, sizeof(float), cudaMemcpyHostToDevice, n->stream) != cudaSuccess)
        rc = MEPI_ERR_CUDA;
    if (!rc) {
        pack_kernel<<<rows / kEwRows, kInPad, 0, n->stream>>>(dx, n_in, dy, nullptr, nullptr, rows, (int)n_rows,
                                                             n->cap, n->X0, n->X0t, n->yb, n->mask);
        rc = enqueue_forward(n, rows, true);
    }
    if (!rc) rc = enqueue_backward(n, rows, n->inv_one, nullptr, nullptr, n->loss_d);
    double l = 0.0;
    if (!rc && (cudaMemcpyAsync(&l, n->loss_d, sizeof(double), cudaMemcpyDeviceToHost, n->stream) != cudaSuccess ||
                (grad && cudaMemcpyAsync(grad, n->g, n->n_params * sizeof(float), cudaMemcpyDeviceToHost,
                                         n->stream) != cudaSuccess)))
        rc = MEPI_ERR_CUDA;
    if (!rc) rc = check_err(n);
    cudaFree(dx);
    if (!rc && loss) *loss = l;
    return rc;
}

int mepi_mlp_train(mepi_mlp* n, int64_t n_rows, const float* x, const float* y, int32_t epochs, int32_t batch,
                   float lr, uint64_t seed, float* loss_hist) {
    if (!n || n_rows < 1 || !x || !y || epochs < 1 || batch < GBM || batch % GBM || batch > kMaxRows ||
        !(lr > 0.f) || n_rows > (int64_t)1 << 30)
        return MEPI_ERR_ARG;
    if (cudaSetDevice(n->device) != cudaSuccess) return MEPI_ERR_CUDA;
    if (int rc = ensure_rows(n, batch)) return rc;
    const int n_in = n->nd.n_in;
    const int64_t steps_per_epoch = (n_rows + batch - 1) / batch;
    const int64_t total = steps_per_epoch * epochs;
    if (total * batch > ((int64_t)1 << 31) - 1) return MEPI_ERR_ARG;
    // the batch order of every step (-1 pads the last batch of an epoch) and 1/rows of each batch
    std::vector<int> order((size_t)(total * batch), -1);
    std::vector<float> inv((size_t)total);
    std::vector<int> perm((size_t)n_rows);
    uint64_t st = seed;
    for (int e = 0; e < epochs; ++e) {
        for (int64_t i = 0; i < n_rows; ++i) perm[i] = (int)i;
        for (int64_t i = n_rows - 1; i > 0; --i) std::swap(perm[i], perm[splitmix(st) % (uint64_t)(i + 1)]);
        for (int64_t s = 0; s < steps_per_epoch; ++s) {
            const int64_t g = e * steps_per_epoch + s;
            const int64_t nv = std::min<int64_t>(batch, n_rows - s * batch);
            for (int64_t r = 0; r < nv; ++r) order[(size_t)(g * batch + r)] = perm[(size_t)(s * batch + r)];
            inv[(size_t)g] = 1.f / (float)nv;
        }
    }
    char* buf = nullptr;
    const size_t bx = (size_t)n_rows * n_in * 4, by = (size_t)n_rows * 4, bo = order.size() * 4, bi = inv.size() * 4,
                 bl = (size_t)total * 4;
    MLP_CK(cudaMalloc(&buf, bx + by + bo + bi + bl + 1024));
    float* dx = reinterpret_cast<float*>(buf);
    float* dy = reinterpret_cast<float*>(buf + bx);
    int* dorder = reinterpret_cast<int*>(buf + bx + by);
    float* dinv = reinterpret_cast<float*>(buf + bx + by + bo);
    float* dloss = reinterpret_cast<float*>(buf + bx + by + bo + bi);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int rc = MEPI_OK;
    if (cudaMemcpyAsync(dx, x, bx, cudaMemcpyHostToDevice, n->stream) != cudaSuccess ||
        cudaMemcpyAsync(dy, y, by, cudaMemcpyHostToDevice, n->stream) != cudaSuccess ||
        cudaMemcpyAsync(dorder, order.data(), bo, cudaMemcpyHostToDevice, n->stream) != cudaSuccess ||
        cudaMemcpyAsync(dinv, inv.data(), bi, cudaMemcpyHostToDevice, n->stream) != cudaSuccess ||
        cudaMemsetAsync(n->step, 0, sizeof(int), n->stream) != cudaSuccess ||
        cudaStreamSynchronize(n->stream) != cudaSuccess)
        rc = MEPI_ERR_CUDA;
    // one step: gather, forward, backward, Adam, BF16 weight copies; captured once
    if (!rc && cudaStreamBeginCapture(n->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = MEPI_ERR_CUDA;
    if (!rc) {
        pack_kernel<<<batch / kEwRows, kInPad, 0, n->stream>>>(dx, n_in, dy, dorder, n->step, batch, 0, n->cap, n->X0,
                                                              n->X0t, n->yb, n->mask);
        int r2 = enqueue_forward(n, batch, true);
        if (!r2) r2 = enqueue_backward(n, batch, dinv, n->step, dloss, nullptr);
        if (!r2) {
            adam_kernel<<<(unsigned)((n->n_params + 255) / 256), 256, 0, n->stream>>>(n->p, n->m, n->v, n->g,
                                                                                     n->n_params, lr, n->step);
            r2 = cudaGetLastError() == cudaSuccess ? refresh_weights(n, n->step) : MEPI_ERR_CUDA;
        }
        const cudaError_t ec = cudaStreamEndCapture(n->stream, &graph);
        rc = r2 ? r2 : (ec != cudaSuccess || !graph) ? MEPI_ERR_CUDA : MEPI_OK;
    }
    if (!rc && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) rc = MEPI_ERR_CUDA;
    for (int64_t s = 0; s < total && !rc; ++s)
        if (cudaGraphLaunch(exec, n->stream) != cudaSuccess) rc = MEPI_ERR_CUDA;
    std::vector<float> hl((size_t)total);
    if (!rc && cudaMemcpyAsync(hl.data(), dloss, bl, cudaMemcpyDeviceToHost, n->stream) != cudaSuccess)
        rc = MEPI_ERR_CUDA;
    if (!rc) rc = check_err(n);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamSynchronize(n->stream);
    cudaFree(buf);
    if (!rc && loss_hist)
        for (int e = 0; e < epochs; ++e) {
            double a = 0.0;
            for (int64_t s = 0; s < steps_per_epoch; ++s) a += hl[(size_t)(e * steps_per_epoch + s)];
            loss_hist[e] = (float)(a / steps_per_epoch);
        }
    return rc;
}

}  // extern "C"
