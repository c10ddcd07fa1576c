// Grouped gather/scatter GEMM on the SIMT pipes.
//
// Every dense translation of the FMM is one of these: for each group g
// (one translation operator A_g) and each pair p of the group,
// D[:, out(p), r] (op)= op(A_g) * B[:, in(p), r] for every right-hand side r.
// Groups are: one per level for the check-to-equivalent products (the
// reference's mat_vec(check_to_equiv, .), cpp/fmm.cpp:195,245,324,376,406),
// one per (level, octant) for M2M / L2L, one per distinct M2L translation
// (level pair + integer offset), and the compressions of the SVD-compressed
// M2L (rectangular operators).  Cell buffers are laid out [cell][rhs][len],
// so a column is len contiguous values: B columns have length k, D columns
// length m.
//
// CTA: 256 threads, tile BM x 64 (BM = 128 or 64: the choice that pads m the
// least), each thread an (BM / 16) x 4 block of outputs.  A launch with too
// few tiles to fill the GPU splits K over blockIdx.z (partial products added
// atomically).  K runs in steps of
// BK through two shared-memory buffers: the next step's global loads are in
// registers while the current step is multiplied, so one barrier per step
// and the load latency overlaps the FMAs.  Shared tiles are stored k-major
// (m / n contiguous, rows padded by 4 to spread the transposing stores over
// the banks) and read as 16-byte vectors.
#pragma once
#include <cuda_runtime.h>

namespace tbem {

constexpr int GM_BN = 64, GM_THREADS = 256;

// GEMM_WAVES: deterministic accumulation -- the groups run in conflict-free
// waves (no output written twice within a wave), each wave with GEMM_ADD.
enum GemmMode { GEMM_STORE = 0, GEMM_ADD = 1, GEMM_ATOMIC = 2, GEMM_WAVES = 3 };

template <typename T>
struct GemmArgs {
    const T* const* A;      // per group, row-major, rows of length lda
    const long* g_pair0;    // per group: first pair
    const int* g_npairs;    // per group: number of pairs
    const int* tile_group;  // per N-tile: group
    const int* tile_col0;   // per N-tile: first logical column within the group
    const int* in_cell;     // per pair
    const int* out_cell;    // per pair
    const T* B;
    T* D;
    int m;      // rows of op(A) = D column length
    int k;      // columns of op(A) = B column length
    int lda;    // row length of the stored A (k, or m when trans)
    int nrhs;
    int trans;  // op(A) = A^T
    int mode;
    int kchunk;  // split K: CTA z covers [z * kchunk, (z + 1) * kchunk) (multiple of BK)
};

template <typename T>
__device__ __forceinline__ void atomic_add_t(T* p, T v);
template <>
__device__ __forceinline__ void atomic_add_t<double>(double* p, double v) { atomicAdd(p, v); }
template <>
__device__ __forceinline__ void atomic_add_t<float>(float* p, float v) { atomicAdd(p, v); }

// K step: 16 for FP32; 8 for FP64 (keeps the two buffers within 48 KB)
template <typename T>
struct GemmK {
    static constexpr int BK = sizeof(T) == 4 ? 16 : 8;
};

// One output tile (column tile `tile`, row tile `mtile`, K split `kz`) of a
// grouped GEMM (the body of grouped_gemm_kernel).
template <typename T, int BM>
__device__ __forceinline__ void gemm_tile(const GemmArgs<T>& a, int tile, int mtile, int kz)
{
    constexpr int BN = GM_BN, BK = GemmK<T>::BK;
    constexpr int TM = BM / 16, TN = BN / 16;  // outputs per thread (rows x columns)
    constexpr int PA = BM + 4, PB = BN + 4;     // padded row lengths of the shared tiles
    constexpr int NA = BM * BK / GM_THREADS;    // A elements loaded per thread per step
    constexpr int NB = BN * BK / GM_THREADS;    // B elements loaded per thread per step
    static_assert(NA >= 1 && NB >= 1, "tile too small for the CTA");
    __shared__ __align__(16) T As[2][BK][PA];
    __shared__ __align__(16) T Bs[2][BK][PB];

    const int g = a.tile_group[tile];
    const int col0 = a.tile_col0[tile];
    const int m0 = mtile * BM;
    if (m0 >= a.m) return;
    const T* __restrict__ A = a.A[g];
    const long pair0 = a.g_pair0[g];
    const int ncols = a.g_npairs[g] * a.nrhs;
    const int M = a.m, K = a.k, lda = a.lda;
    const long ldb = (long)a.nrhs * K;  // cell stride in B
    const long ldd = (long)a.nrhs * M;  // cell stride in D
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;

    // B: this thread's gathered columns (fixed for the whole K loop).  Element
    // e = tid + i * 256 of a step is column e / BK, depth e % BK.
    const T* bcol[NB];
    int bk[NB], bj[NB];
#pragma unroll
    for (int i = 0; i < NB; i++) {
        const int e = tid + i * GM_THREADS;
        bj[i] = e / BK;
        bk[i] = e % BK;
        const int c = col0 + bj[i];
        bcol[i] = nullptr;
        if (c < ncols) {
            const int p = c / a.nrhs, r = c % a.nrhs;
            bcol[i] = a.B + (long)a.in_cell[pair0 + p] * ldb + (long)r * K;
        }
    }
    // A: element e of a step is (row e / BK, depth e % BK) without transpose
    // (k contiguous in memory), (depth e / BM, row e % BM) with it
    int am[NA], ak[NA];
#pragma unroll
    for (int i = 0; i < NA; i++) {
        const int e = tid + i * GM_THREADS;
        if (!a.trans) { am[i] = e / BK; ak[i] = e % BK; }
        else { ak[i] = e / BM; am[i] = e % BM; }
    }

    T ra[NA], rb[NB];
    // this CTA's K range (split K: the partial products meet in GEMM_ATOMIC)
    const int kb = kz * a.kchunk;
    const int kend = min(K, kb + a.kchunk);
    auto load = [&](int k0) {
#pragma unroll
        for (int i = 0; i < NA; i++) {
            const int gm = m0 + am[i], gk = k0 + ak[i];
            T v = T(0);
            if (gm < M && gk < kend) v = a.trans ? A[(long)gk * lda + gm] : A[(long)gm * lda + gk];
            ra[i] = v;
        }
#pragma unroll
        for (int i = 0; i < NB; i++) {
            const int gk = k0 + bk[i];
            rb[i] = (bcol[i] && gk < kend) ? bcol[i][gk] : T(0);
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int i = 0; i < NA; i++) As[buf][ak[i]][am[i]] = ra[i];
#pragma unroll
        for (int i = 0; i < NB; i++) Bs[buf][bk[i]][bj[i]] = rb[i];
    };

    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) acc[i][j] = T(0);

    const int nk = (kend - kb + BK - 1) / BK;
    load(kb);
    store(0);
    __syncthreads();
    for (int kt = 0; kt < nk; kt++) {
        const int buf = kt & 1;
        if (kt + 1 < nk) load(kb + (kt + 1) * BK);
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            T av[TM], bv[TN];
#pragma unroll
            for (int i = 0; i < TM; i += 4) {
                if constexpr (sizeof(T) == 4) {
                    const float4 v = *reinterpret_cast<const float4*>(&As[buf][kk][ty * TM + i]);
                    av[i] = v.x; av[i + 1] = v.y; av[i + 2] = v.z; av[i + 3] = v.w;
                } else {
                    const double2 v0 = *reinterpret_cast<const double2*>(&As[buf][kk][ty * TM + i]);
                    const double2 v1 = *reinterpret_cast<const double2*>(&As[buf][kk][ty * TM + i + 2]);
                    av[i] = v0.x; av[i + 1] = v0.y; av[i + 2] = v1.x; av[i + 3] = v1.y;
                }
            }
            if constexpr (sizeof(T) == 4) {
                const float4 v = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * TN]);
                bv[0] = v.x; bv[1] = v.y; bv[2] = v.z; bv[3] = v.w;
            } else {
                const double2 v0 = *reinterpret_cast<const double2*>(&Bs[buf][kk][tx * TN]);
                const double2 v1 = *reinterpret_cast<const double2*>(&Bs[buf][kk][tx * TN + 2]);
                bv[0] = v0.x; bv[1] = v0.y; bv[2] = v1.x; bv[3] = v1.y;
            }
#pragma unroll
            for (int i = 0; i < TM; i++)
#pragma unroll
                for (int j = 0; j < TN; j++) acc[i][j] += av[i] * bv[j];
        }
        if (kt + 1 < nk) store(buf ^ 1);
        __syncthreads();
    }
    // resolve the output columns before the first store (no load behind a store)
    T* dcols[TN];
#pragma unroll
    for (int j = 0; j < TN; j++) {
        const int c = col0 + tx * TN + j;
        dcols[j] = nullptr;
        if (c < ncols) {
            const int p = c / a.nrhs, r = c % a.nrhs;
            dcols[j] = a.D + (long)a.out_cell[pair0 + p] * ldd + (long)r * M;
        }
    }
#pragma unroll
    for (int j = 0; j < TN; j++) {
        T* dcol = dcols[j];
        if (!dcol) continue;
#pragma unroll
        for (int i = 0; i < TM; i++) {
            const int gm = m0 + ty * TM + i;
            if (gm >= M) continue;
            if (a.mode == GEMM_STORE) dcol[gm] = acc[i][j];
            else if (a.mode == GEMM_ADD) dcol[gm] += acc[i][j];
            else atomic_add_t<T>(&dcol[gm], acc[i][j]);
        }
    }
}

template <typename T, int BM>
__global__ void __launch_bounds__(GM_THREADS) grouped_gemm_kernel(const GemmArgs<T> a)
{
    gemm_tile<T, BM>(a, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Row tile for m rows: the one that pads m the least (128 on a tie).
inline int gemm_bm(int m)
{
    const int p128 = (m + 127) / 128 * 128, p64 = (m + 63) / 64 * 64;
    return p64 < p128 ? 64 : 128;
}

}  // namespace tbem
