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
// Precision: the plan is built in FP64.  The FP64 form keeps G2 in FP64 for all
// blocks.  The mixed form keeps all blocks in FP32 (nbz-term sums of FP32
// values, about 1e-7 relative) plus block 0 (H) in FP64 for the FP64 eigenpair
// refinement.
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

// G1[qx][iy][iz][e] = sum_ix phase(kx, Rx0 + ix) box[ix][iy][iz][e],  e = blk * NN + pair
__global__ void sep_stage_a(const cplx<double>* __restrict__ box, cplx<double>* __restrict__ G1, int EL, int nbx,
                            int nby, int nbz, int rx0, int n1) {
    const int yz = blockIdx.y, qx = blockIdx.z;
    const double kx = mp_coord(qx, n1);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < EL; e += gridDim.x * blockDim.x) {
        cplx<double> acc = mk(0.0, 0.0);
        for (int ix = 0; ix < nbx; ++ix)
            fma_c(acc, phase(kx, rx0 + ix), box[((size_t)ix * nby * nbz + yz) * EL + e]);
        G1[((size_t)qx * nby * nbz + yz) * EL + e] = acc;
    }
}

// G2[qx][qy][iz][e] = sum_iy phase(ky, Ry0 + iy) G1[qx][iy][iz][e]; the first
// nbd blocks go to G2d (FP64), all blocks to G2f (FP32) when it is allocated.
__global__ void sep_stage_b(const cplx<double>* __restrict__ G1, cplx<double>* __restrict__ G2d,
                            cplx<float>* __restrict__ G2f, int NN, int nbk, int nbd, int nby, int nbz, int ry0, int n1,
                            int n2) {
    const int iz = blockIdx.y % nbz, qy = blockIdx.y / nbz, qx = blockIdx.z;
    const double ky = mp_coord(qy, n2);
    const int EL = nbk * NN;
    const size_t cell = ((size_t)qx * n2 + qy) * nbz + iz;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < EL; e += gridDim.x * blockDim.x) {
        cplx<double> acc = mk(0.0, 0.0);
        for (int iy = 0; iy < nby; ++iy)
            fma_c(acc, phase(ky, ry0 + iy), G1[(((size_t)qx * nby + iy) * nbz + iz) * EL + e]);
        if (e < nbd * NN) G2d[cell * nbd * NN + e] = acc;
        if (G2f) G2f[cell * EL + e] = mk((float)acc.re, (float)acc.im);
    }
}

constexpr int kSepItems = 2;  // k-points per CTA in the per-k stages

__device__ __forceinline__ void item_coords(const KRange& kr, int64_t i, int q[3], double k[3]) {
    const int64_t ki = k_of(kr, i);
    q[0] = (int)(ki % kr.mp[0]);
    q[1] = (int)((ki / kr.mp[0]) % kr.mp[1]);
    q[2] = (int)(ki / ((int64_t)kr.mp[0] * kr.mp[1]));
    for (int a = 0; a < 3; ++a) k[a] = mp_coord(q[a], kr.mp[a]);
}

// W[i][blk][pair] for all stack blocks: X_b = sum_iz phase(kz) G2[qx][qy][iz][b][pair]
// accumulated in TG, then the tight-binding epilogue in FP64.
template <typename T, typename TG, int NB>
__global__ void __launch_bounds__(256) sep_w_kernel(DevModel m, KRange kr, const cplx<TG>* __restrict__ G2, int nbz,
                                                    int rz0, cplx<T>* __restrict__ W) {
    const int NN = m.N * m.N;
    __shared__ cplx<TG> ph[kSepItems][32];
    __shared__ double ks[kSepItems][3];
    __shared__ int qs[kSepItems][2];
    const int64_t i0 = (int64_t)blockIdx.x * kSepItems;
    if (threadIdx.x < kSepItems) {
        const int64_t i = i0 + threadIdx.x;
        int q[3] = {0, 0, 0};
        double k[3] = {0.0, 0.0, 0.0};
        if (i < kr.count) item_coords(kr, i, q, k);
        ks[threadIdx.x][0] = k[0]; ks[threadIdx.x][1] = k[1]; ks[threadIdx.x][2] = k[2];
        qs[threadIdx.x][0] = q[0]; qs[threadIdx.x][1] = q[1];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kSepItems * 32; e += blockDim.x) {
        const int it = e / 32, iz = e % 32;
        cplx<double> p = iz < nbz ? phase(ks[it][2], rz0 + iz) : mk(0.0, 0.0);
        ph[it][iz] = mk((TG)p.re, (TG)p.im);
    }
    __syncthreads();
    for (int it = 0; it < kSepItems; ++it) {
        const int64_t i = i0 + it;
        if (i >= kr.count) break;
        const cplx<TG>* g = G2 + ((size_t)qs[it][0] * kr.mp[1] + qs[it][1]) * nbz * NB * NN;
        const double k[3] = {ks[it][0], ks[it][1], ks[it][2]};
        for (int pair = threadIdx.x; pair < NN; pair += blockDim.x) {
            cplx<TG> acc[NB];
#pragma unroll
            for (int b = 0; b < NB; ++b) acc[b] = mk((TG)0, (TG)0);
            for (int iz = 0; iz < nbz; ++iz) {
                const cplx<TG> p = ph[it][iz];
                const cplx<TG>* gz = g + (size_t)iz * NB * NN + pair;
#pragma unroll
                for (int b = 0; b < NB; ++b) fma_c(acc[b], p, gz[(size_t)b * NN]);
            }
            cplx<double> X[NB];
#pragma unroll
            for (int b = 0; b < NB; ++b) X[b] = mk((double)acc[b].re, (double)acc[b].im);
            ft_epilogue<T, NB>(m, k, pair, X, W + (size_t)i * NB * NN, NN);
        }
    }
}

// H64[i][pair] = psi * sum_iz phase(kz) G2d[qx][qy][iz][0][pair]
__global__ void __launch_bounds__(256) sep_h64_kernel(const cplx<double>* __restrict__ G2, KRange kr, int N, int nbd,
                                                      int nbz, int rz0, const double* __restrict__ tau,
                                                      cplx<double>* __restrict__ H64) {
    const int NN = N * N;
    __shared__ cplx<double> ph[kSepItems][32];
    __shared__ double ks[kSepItems][3];
    __shared__ int qs[kSepItems][2];
    const int64_t i0 = (int64_t)blockIdx.x * kSepItems;
    if (threadIdx.x < kSepItems) {
        const int64_t i = i0 + threadIdx.x;
        int q[3] = {0, 0, 0};
        double k[3] = {0.0, 0.0, 0.0};
        if (i < kr.count) item_coords(kr, i, q, k);
        ks[threadIdx.x][0] = k[0]; ks[threadIdx.x][1] = k[1]; ks[threadIdx.x][2] = k[2];
        qs[threadIdx.x][0] = q[0]; qs[threadIdx.x][1] = q[1];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kSepItems * 32; e += blockDim.x) {
        const int it = e / 32, iz = e % 32;
        ph[it][iz] = iz < nbz ? phase(ks[it][2], rz0 + iz) : mk(0.0, 0.0);
    }
    __syncthreads();
    for (int it = 0; it < kSepItems; ++it) {
        const int64_t i = i0 + it;
        if (i >= kr.count) break;
        const cplx<double>* g = G2 + ((size_t)qs[it][0] * kr.mp[1] + qs[it][1]) * nbz * nbd * NN;
        for (int pair = threadIdx.x; pair < NN; pair += blockDim.x) {
            cplx<double> acc = mk(0.0, 0.0);
            for (int iz = 0; iz < nbz; ++iz) fma_c(acc, ph[it][iz], g[(size_t)iz * nbd * NN + pair]);
            if (tau) {
                const int n = pair / N, mm = pair % N;
                const double x = ks[it][0] * (tau[mm * 3] - tau[n * 3]) + ks[it][1] * (tau[mm * 3 + 1] - tau[n * 3 + 1]) +
                                 ks[it][2] * (tau[mm * 3 + 2] - tau[n * 3 + 2]);
                double s, c;
                sincospi(2.0 * x, &s, &c);
                acc = mk(c, s) * acc;
            }
            H64[(size_t)i * NN + pair] = acc;
        }
    }
}

}  // namespace

int sep_plan_build(SepPlan& p, const DevModel& m, const double* R_host, const cplx<double>* S_host, const int mp[3],
                   bool fp64, cudaStream_t s) {
    if (p.ready && p.fp64 == fp64 && p.mp[0] == mp[0] && p.mp[1] == mp[1] && p.mp[2] == mp[2]) return 0;
    sep_plan_free(p);
    int lo[3] = {1 << 30, 1 << 30, 1 << 30}, hi[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    for (int r = 0; r < m.nR; ++r)
        for (int a = 0; a < 3; ++a) {
            const double v = R_host[3 * r + a];
            if (std::fabs(v - std::rint(v)) > 1e-9 || std::fabs(v) > 1e6) return 1;
            lo[a] = std::min(lo[a], (int)std::lrint(v));
            hi[a] = std::max(hi[a], (int)std::lrint(v));
        }
    const int nb[3] = {hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, hi[2] - lo[2] + 1};
    if (nb[0] > 32 || nb[1] > 32 || nb[2] > 32) return 1;
    const int NN = m.N * m.N, nbk = m.nb, EL = nbk * NN;
    const int nbd = fp64 ? nbk : 1;
    const size_t box = (size_t)nb[0] * nb[1] * nb[2];
    const size_t slabs = (size_t)mp[0] * mp[1] * nb[2];
    const size_t g2d_bytes = slabs * nbd * NN * sizeof(cplx<double>);
    const size_t g2f_bytes = fp64 ? 0 : slabs * EL * sizeof(cplx<float>);
    const size_t g1_bytes = (size_t)mp[0] * nb[1] * nb[2] * EL * sizeof(cplx<double>);
    const size_t box_bytes = box * EL * sizeof(cplx<double>);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 2;
    // the slabs stay resident for the run; leave room for the per-chunk buffers
    if (g2d_bytes + g2f_bytes + g1_bytes + box_bytes > free_b / 2) return 1;
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
    cplx<double>* dbox = nullptr;
    cplx<double>* G1 = nullptr;
    auto cleanup = [&](int rc) {
        if (dbox) cudaFree(dbox);
        if (G1) cudaFree(G1);
        if (rc) sep_plan_free(p);
        return rc;
    };
    if (cudaMalloc(&dbox, box_bytes) != cudaSuccess) return cleanup(3);
    if (cudaMalloc(&G1, g1_bytes) != cudaSuccess) return cleanup(3);
    if (cudaMalloc(&p.G2d, g2d_bytes) != cudaSuccess) return cleanup(3);
    if (!fp64 && cudaMalloc(&p.G2f, g2f_bytes) != cudaSuccess) return cleanup(3);
    if (cudaMemcpyAsync(dbox, hb.data(), box_bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) return cleanup(2);
    dim3 ga((EL + 255) / 256, nb[1] * nb[2], mp[0]);
    sep_stage_a<<<ga, 256, 0, s>>>(dbox, G1, EL, nb[0], nb[1], nb[2], lo[0], mp[0]);
    dim3 gb((EL + 255) / 256, mp[1] * nb[2], mp[0]);
    sep_stage_b<<<gb, 256, 0, s>>>(G1, p.G2d, p.G2f, NN, nbk, nbd, nb[1], nb[2], lo[1], mp[0], mp[1]);
    if (cudaGetLastError() != cudaSuccess) return cleanup(2);
    // the temporaries are freed only after the stage kernels have run
    if (cudaStreamSynchronize(s) != cudaSuccess) return cleanup(2);
    for (int a = 0; a < 3; ++a) {
        p.mp[a] = mp[a];
        p.lo[a] = lo[a];
        p.nb[a] = nb[a];
    }
    p.N = m.N;
    p.nbk = nbk;
    p.nbd = nbd;
    p.fp64 = fp64;
    p.tau = m.has_tau ? m.tau : nullptr;
    p.h2d_bytes = box_bytes;
    p.ready = true;
    return cleanup(0);
}

void sep_plan_free(SepPlan& p) {
    if (p.G2d) cudaFree(p.G2d);
    if (p.G2f) cudaFree(p.G2f);
    p = SepPlan();
}

cudaError_t launch_sep_h64(const SepPlan& p, const KRange& kr, cplx<double>* H64, cudaStream_t s) {
    if (kr.count <= 0) return cudaSuccess;
    const unsigned grid = (unsigned)((kr.count + kSepItems - 1) / kSepItems);
    sep_h64_kernel<<<grid, 256, 0, s>>>(p.G2d, kr, p.N, p.nbd, p.nb[2], p.lo[2], p.tau, H64);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_sep_w(const SepPlan& p, const DevModel& m, const KRange& kr, cplx<T>* W, cudaStream_t s) {
    if (kr.count <= 0) return cudaSuccess;
    const unsigned grid = (unsigned)((kr.count + kSepItems - 1) / kSepItems);
    const int threads = m.N <= 8 ? 64 : 256;
    if (p.fp64) {
        if (m.nb == 10)
            sep_w_kernel<T, double, 10><<<grid, threads, 0, s>>>(m, kr, p.G2d, p.nb[2], p.lo[2], W);
        else
            sep_w_kernel<T, double, 4><<<grid, threads, 0, s>>>(m, kr, p.G2d, p.nb[2], p.lo[2], W);
    } else {
        if (sizeof(T) == 8) return cudaErrorInvalidValue;  // FP64 output needs the FP64 slabs
        if (m.nb == 10)
            sep_w_kernel<T, float, 10><<<grid, threads, 0, s>>>(m, kr, p.G2f, p.nb[2], p.lo[2], W);
        else
            sep_w_kernel<T, float, 4><<<grid, threads, 0, s>>>(m, kr, p.G2f, p.nb[2], p.lo[2], W);
    }
    return cudaGetLastError();
}

template cudaError_t launch_sep_w<double>(const SepPlan&, const DevModel&, const KRange&, cplx<double>*, cudaStream_t);
template cudaError_t launch_sep_w<float>(const SepPlan&, const DevModel&, const KRange&, cplx<float>*, cudaStream_t);

}  // namespace mepi
