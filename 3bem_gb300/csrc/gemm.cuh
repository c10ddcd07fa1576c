// Grouped gather/scatter GEMM on the SIMT pipes.
//
// Every dense translation of the FMM is one of these: for each group g
// (one translation operator A_g, n x n row-major) and each pair p of the
// group, D[:, out(p), r] (op)= A_g * B[:, in(p), r] for every right-hand
// side r.  Groups are: one per level for the check-to-equivalent products
// (the reference's mat_vec(check_to_equiv, .), cpp/fmm.cpp:195,245,324,376,
// 406), one per (level, octant) for M2M / L2L, one per distinct M2L
// translation (level pair + integer offset).  Cell buffers are laid out
// [cell][rhs][n], so a column is n contiguous values.
//
// CTA tile 64 x 64 x 16, 256 threads, 4 x 4 outputs per thread.
#pragma once
#include <cuda_runtime.h>

namespace tbem {

constexpr int GM_BM = 64, GM_BN = 64, GM_BK = 16, GM_THREADS = 256;

// GEMM_WAVES: deterministic accumulation -- the groups run in conflict-free
// waves (no output written twice within a wave), each wave with GEMM_ADD.
enum GemmMode { GEMM_STORE = 0, GEMM_ADD = 1, GEMM_ATOMIC = 2, GEMM_WAVES = 3 };

template <typename T>
struct GemmArgs {
    const T* const* A;      // per group, n x n row-major
    const long* g_pair0;    // per group: first pair
    const int* g_npairs;    // per group: number of pairs
    const int* tile_group;  // per N-tile: group
    const int* tile_col0;   // per N-tile: first logical column within the group
    const int* in_cell;     // per pair
    const int* out_cell;    // per pair
    const T* B;
    T* D;
    int n;
    int nrhs;
    int trans;  // use A^T
    int mode;
};

template <typename T>
__device__ __forceinline__ void atomic_add_t(T* p, T v);
template <>
__device__ __forceinline__ void atomic_add_t<double>(double* p, double v) { atomicAdd(p, v); }
template <>
__device__ __forceinline__ void atomic_add_t<float>(float* p, float v) { atomicAdd(p, v); }

template <typename T>
__global__ void __launch_bounds__(GM_THREADS) grouped_gemm_kernel(const GemmArgs<T> a)
{
    __shared__ T As[GM_BK][GM_BM + 1];
    __shared__ T Bs[GM_BK][GM_BN + 1];
    const int tile = blockIdx.x;
    const int g = a.tile_group[tile];
    const int col0 = a.tile_col0[tile];
    const int m0 = blockIdx.y * GM_BM;
    if (m0 >= a.n) return;
    const T* A = a.A[g];
    const long pair0 = a.g_pair0[g];
    const int ncols = a.g_npairs[g] * a.nrhs;
    const int n = a.n;
    const long ldc = (long)a.nrhs * n;  // cell stride in B and D

    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    // column pointers of the B tile handled by this thread when loading
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0;

    for (int k0 = 0; k0 < n; k0 += GM_BK) {
        // A tile: 64 rows x 16 k
#pragma unroll
        for (int i = 0; i < (GM_BM * GM_BK) / GM_THREADS; i++) {
            int idx = tid + i * GM_THREADS;
            int m, k;
            if (!a.trans) { m = idx / GM_BK; k = idx % GM_BK; }
            else { k = idx / GM_BM; m = idx % GM_BM; }
            int gm = m0 + m, gk = k0 + k;
            T v = 0;
            if (gm < n && gk < n) v = a.trans ? A[(long)gk * n + gm] : A[(long)gm * n + gk];
            As[k][m] = v;
        }
        // B tile: 64 gathered columns x 16 k
#pragma unroll
        for (int i = 0; i < (GM_BN * GM_BK) / GM_THREADS; i++) {
            int idx = tid + i * GM_THREADS;
            int j = idx / GM_BK, k = idx % GM_BK;
            int c = col0 + j, gk = k0 + k;
            T v = 0;
            if (c < ncols && gk < n) {
                int p = c / a.nrhs, r = c % a.nrhs;
                long cell = a.in_cell[pair0 + p];
                v = a.B[cell * ldc + (long)r * n + gk];
            }
            Bs[k][j] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GM_BK; kk++) {
            T av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; i++) av[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; j++) bv[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] += av[i] * bv[j];
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        int c = col0 + tx * 4 + j;
        if (c >= ncols) continue;
        int p = c / a.nrhs, r = c % a.nrhs;
        long cell = a.out_cell[pair0 + p];
        T* dcol = a.D + cell * ldc + (long)r * n;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            int gm = m0 + ty * 4 + i;
            if (gm >= n) continue;
            if (a.mode == GEMM_STORE) dcol[gm] = acc[i][j];
            else if (a.mode == GEMM_ADD) dcol[gm] += acc[i][j];
            else atomic_add_t<T>(&dcol[gm], acc[i][j]);
        }
    }
}

}  // namespace tbem
