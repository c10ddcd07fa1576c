// Host-side launcher of the obs-owner evaluation kernels (eval.cuh).
#pragma once
#include <cuda_runtime.h>
#include "eval.cuh"

namespace tbem {

struct EvalLaunch {
    int kid;
    bool trans;
    bool tgt_surf;
    bool src_surf;
    int n_items;
    int tpt = 4;  // threads per target (2, 4 or 8 for the point-to-point pass, 1, 2 or 4
                  // for points to a check surface; 4 otherwise)
};

// One function per kernel id (eval_k<id>.cu) so that the instantiations
// compile in parallel.
cudaError_t launch_eval_k0(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k1(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k2(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k3(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k4(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k5(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k6(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
// 2D kernels (FP64 only)
cudaError_t launch_eval_k16(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k17(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k18(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k19(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k20(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k21(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k22(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);
cudaError_t launch_eval_k23(const EvalLaunch&, const void* args, bool fp32, cudaStream_t);

// rhs chunk per launch (the kernel keeps NR x R accumulators per thread)
constexpr int EVAL_NR = 4;
// FP32 scalar kernels with point sources, not transposed: 16 right-hand
// sides per launch (the kernel value is shared by all of them)
constexpr int EVAL_NR_WIDE = 16;

// Right-hand sides one launch of the evaluation kernel handles when
// `remaining` are left from the launch's first one.
inline int eval_rhs_block(int kid, bool fp32, bool trans, bool src_surf, int remaining)
{
    if (remaining <= 1) return 1;
    if (fp32 && kernel_dim(kid) == 1 && kernel_space_dim(kid) == 3 && !trans && !src_surf &&
        remaining >= EVAL_NR_WIDE)
        return EVAL_NR_WIDE;
    return EVAL_NR;
}

template <typename T>
inline cudaError_t launch_eval(const EvalLaunch& L, const EvalArgs<T>& a, cudaStream_t s)
{
    const bool fp32 = sizeof(T) == 4;
    switch (L.kid) {
    case 0: return launch_eval_k0(L, &a, fp32, s);
    case 1: return launch_eval_k1(L, &a, fp32, s);
    case 2: return launch_eval_k2(L, &a, fp32, s);
    case 3: return launch_eval_k3(L, &a, fp32, s);
    case 4: return launch_eval_k4(L, &a, fp32, s);
    case 5: return launch_eval_k5(L, &a, fp32, s);
    case 6: return launch_eval_k6(L, &a, fp32, s);
    case 16: return launch_eval_k16(L, &a, fp32, s);
    case 17: return launch_eval_k17(L, &a, fp32, s);
    case 18: return launch_eval_k18(L, &a, fp32, s);
    case 19: return launch_eval_k19(L, &a, fp32, s);
    case 20: return launch_eval_k20(L, &a, fp32, s);
    case 21: return launch_eval_k21(L, &a, fp32, s);
    case 22: return launch_eval_k22(L, &a, fp32, s);
    case 23: return launch_eval_k23(L, &a, fp32, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace tbem
