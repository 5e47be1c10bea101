// Host-side plan of the tensor-core Fourier GEMM (ft_tc.cu).
#pragma once
#include <cuda.h>
#include <cuda_fp16.h>

#include "mepi_internal.cuh"

namespace mepi {

constexpr float kTcAScale = 4096.0f;  // 2^12 scale of the phase operand
enum { MEPI_TC_NOMEM = 3, MEPI_TC_CUDA = 2 };

struct TcPlan {
    int N = 0, nb = 0, nR = 0, PT = 0, TN = 0, n_tiles = 0, Kp = 0;
    size_t ncolp = 0;
    int64_t rows = 0, rows_cap = 0;
    double C[9] = {0};
    float inv_scale[10] = {0};
    __half *Bh = nullptr, *Bl = nullptr, *Ah = nullptr, *Al = nullptr;
    const double* tau = nullptr;   // device (N,3) or nullptr
    const double* R = nullptr;     // device (nR,3)
    int* err = nullptr;            // device flag: a bounded wait timed out
    CUtensorMap tmAh, tmAl, tmBh, tmBl;
    bool ready() const { return Bh != nullptr; }
};

// Split the FP64 stack S[R][pair][blk] into the B' hi/lo operands (host work
// once per model) and build their tensor maps.  Returns 0 or a MEPI_ERR_* code.
int tc_plan_init(TcPlan& p, const DevModel& m, const cplx<double>* S_host);
// Make room for A' of rows_needed k-points (rounded up to 128).
int tc_plan_rows(TcPlan& p, int64_t rows_needed);
void tc_plan_free(TcPlan& p);
cudaError_t launch_phase_split(const TcPlan& p, const KRange& kr, cudaStream_t s);
cudaError_t launch_ft_tc(const TcPlan& p, const KRange& kr, cplx<float>* W, cudaStream_t s);

}  // namespace mepi
