// Instantiates the evaluation kernels of one kernel id (EVAL_KID); with
// EVAL_FP64_ONLY (the 2D kernels, which have the plain FP64 form only) the
// FP32 variants are not built and asking for them is an error.
#include "eval_launch.h"

namespace tbem {

namespace {
template <typename T, bool TR, bool TS, bool SS, int TPT>
void go_tpt(int nr, int n_items, const EvalArgs<T>& a, cudaStream_t s)
{
    if (nr == 1) {
        eval_kernel<EVAL_KID, TR, T, 1, TS, SS, TPT><<<n_items, EVAL_THREADS, 0, s>>>(a);
        return;
    }
    if constexpr (sizeof(T) == 4 && kernel_dim(EVAL_KID) == 1 && kernel_space_dim(EVAL_KID) == 3 &&
                  !TR && !SS) {
        if (nr == EVAL_NR_WIDE) {
            eval_wide_kernel<EVAL_KID, TS, TPT, EVAL_NR_WIDE><<<n_items, EVAL_THREADS / 2, 0, s>>>(a);
            return;
        }
    }
    eval_kernel<EVAL_KID, TR, T, EVAL_NR, TS, SS, TPT><<<n_items, EVAL_THREADS, 0, s>>>(a);
}

template <typename T, bool TR, bool TS, bool SS>
cudaError_t go(int nr, int n_items, int tpt, const void* args, cudaStream_t s)
{
    const EvalArgs<T>& a = *static_cast<const EvalArgs<T>*>(args);
    if (n_items <= 0) return cudaSuccess;
    // the point-to-point pass (2, 4, 8) and the points-to-check-surface pass
    // (1, 2, 4) have autotuned variants; every other pass uses 4
    if (!TR && !TS && !SS && tpt == 2) go_tpt<T, TR, TS, SS, 2>(nr, n_items, a, s);
    else if (!TR && !TS && !SS && tpt == 8) go_tpt<T, TR, TS, SS, 8>(nr, n_items, a, s);
    else if (!TR && TS && !SS && tpt == 1) go_tpt<T, TR, TS, SS, 1>(nr, n_items, a, s);
    else if (!TR && TS && !SS && tpt == 2) go_tpt<T, TR, TS, SS, 2>(nr, n_items, a, s);
    else go_tpt<T, TR, TS, SS, 4>(nr, n_items, a, s);
    return cudaGetLastError();
}

template <typename T>
cudaError_t go_t(const EvalLaunch& L, const void* args, cudaStream_t s)
{
    const EvalArgs<T>& a = *static_cast<const EvalArgs<T>*>(args);
    const int nr = eval_rhs_block(L.kid, sizeof(T) == 4, L.trans, L.src_surf, a.nrhs - a.rhs0);
    const int idx = (L.trans ? 4 : 0) + (L.tgt_surf ? 2 : 0) + (L.src_surf ? 1 : 0);
    switch (idx) {
    case 0: return go<T, false, false, false>(nr, L.n_items, L.tpt, args, s);
    case 1: return go<T, false, false, true>(nr, L.n_items, 4, args, s);
    case 2: return go<T, false, true, false>(nr, L.n_items, L.tpt, args, s);
    case 3: return go<T, false, true, true>(nr, L.n_items, 4, args, s);
    case 4: return go<T, true, false, false>(nr, L.n_items, 4, args, s);
    case 5: return go<T, true, false, true>(nr, L.n_items, 4, args, s);
    case 6: return go<T, true, true, false>(nr, L.n_items, 4, args, s);
    default: return go<T, true, true, true>(nr, L.n_items, 4, args, s);
    }
}
}  // namespace

#define TBEM_CAT2(a, b) a##b
#define TBEM_CAT(a, b) TBEM_CAT2(a, b)
cudaError_t TBEM_CAT(launch_eval_k, EVAL_KID)(const EvalLaunch& L, const void* args, bool fp32,
                                              cudaStream_t s)
{
#ifdef EVAL_FP64_ONLY
    if (fp32) return cudaErrorInvalidValue;
    return go_t<double>(L, args, s);
#else
    return fp32 ? go_t<float>(L, args, s) : go_t<double>(L, args, s);
#endif
}

}  // namespace tbem
