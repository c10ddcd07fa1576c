// FMM plan construction and the apply sequences (forward and transposed),
// for the plain FP64 form and the precision (mixed) form.
//
// Reference schedule (execute_tasks, cpp/fmm.cpp:445-548): P2M, M2M, P2P,
// M2P, P2L, M2L, L2L, L2P.  Here the per-task C2E products are hoisted to
// one grouped GEMM per level (linearity: the reference adds
// C2E_l (K m) for every pair, this adds the K m first), the M2M / L2L / M2L
// kernel matrices are deduplicated by translation (all cells of one level
// share their half widths, cpp/geometry.cpp:20-28), and the levels run
// bottom-up / top-down instead of the serial post-/pre-order walks
// (cpp/fmm.cpp:467-482, 523-538), which respects the same dependencies.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <tuple>

#include "nearfield.h"
#include "plan.h"

namespace tbem {

void check_cuda(cudaError_t e, const char* what, const char* file, int line)
{
    if (e == cudaSuccess) return;
    cudaGetLastError();
    throw Error(e == cudaErrorMemoryAllocation ? TBEM_ERR_ALLOC : TBEM_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e) + " (" + file + ":" +
                    std::to_string(line) + ")");
}
void check_cublas(cublasStatus_t e, const char* what, const char* file, int line)
{
    if (e == CUBLAS_STATUS_SUCCESS) return;
    throw Error(TBEM_ERR_CUDA, std::string(what) + ": cuBLAS status " + std::to_string((int)e) +
                                   " (" + file + ":" + std::to_string(line) + ")");
}
void check_cusolver(cusolverStatus_t e, const char* what, const char* file, int line)
{
    if (e == CUSOLVER_STATUS_SUCCESS) return;
    throw Error(TBEM_ERR_CUDA, std::string(what) + ": cuSOLVER status " +
                                   std::to_string((int)e) + " (" + file + ":" +
                                   std::to_string(line) + ")");
}

// ------------------------------------------------------------------ helpers

void TaskSet::add(long target, int count, const double* org,
                  const std::vector<std::pair<long, int>>& srcs, int targets_per_cta,
                  const std::vector<int>& near)
{
    int pre = 0;
    for (auto& s : srcs) pre += std::max(s.second, 0);
    if (count <= 0 || pre == 0) return;
    const int t = (int)tgt.size();
    tgt.push_back(target);
    tgt_count.push_back(count);
    origin.insert(origin.end(), org, org + 3);
    pre = 0;
    for (size_t i = 0; i < srcs.size(); i++) {
        const auto& s = srcs[i];
        if (s.second <= 0) continue;
        if (!near.empty()) {
            blk_near.resize(blk.size(), 0);  // earlier tasks without flags
            blk_near.push_back(near[i]);
        }
        blk.push_back(s.first);
        blk_count.push_back(s.second);
        blk_prefix.push_back(pre);
        pre += s.second;
    }
    src_ptr.push_back((int)blk.size());
    n_pairs += (long)count * pre;
    for (int st = 0; st < count; st += targets_per_cta) {
        item_task.push_back(t);
        item_start.push_back(st);
    }
}

void TaskSet::upload()
{
    d_tgt.upload(tgt);
    d_tgt_count.upload(tgt_count);
    d_origin.upload(origin);
    d_src_ptr.upload(src_ptr);
    d_blk.upload(blk);
    d_blk_count.upload(blk_count);
    d_blk_prefix.upload(blk_prefix);
    if (!blk_near.empty()) {
        blk_near.resize(blk.size(), 0);
        d_blk_near.upload(blk_near);
    }
    d_item_task.upload(item_task);
    d_item_start.upload(item_start);
}

void GemmSet::add_group(long a_off, const std::vector<std::pair<int, int>>& pairs)
{
    if (pairs.empty()) return;
    A_off.push_back(a_off);
    pair0.push_back((long)in_cell.size());
    npairs.push_back((int)pairs.size());
    for (auto& p : pairs) {
        in_cell.push_back(p.first);
        out_cell.push_back(p.second);
    }
}

void GemmSet::upload(const void* pool, size_t esz)
{
    std::vector<const void*> ptrs(A_off.size());
    for (size_t g = 0; g < A_off.size(); g++)
        ptrs[g] = static_cast<const char*>(pool) + A_off[g] * esz;
    d_A.upload(ptrs);
    d_pair0.upload(pair0);
    d_npairs.upload(npairs);
    d_in.upload(in_cell);
    d_out.upload(out_cell);
    tiles.clear();
}

// Greedy wave assignment: a group goes one wave after the latest wave that
// already writes any of its output cells, so no wave writes a cell twice.
void GemmSet::build_waves()
{
    int max_cell = 0;
    for (int c : out_cell) max_cell = std::max(max_cell, c);
    std::vector<int> last(max_cell + 1, -1);
    wave_of.assign(npairs.size(), 0);
    n_waves = 0;
    for (size_t g = 0; g < npairs.size(); g++) {
        int w = 0;
        for (long p = pair0[g]; p < pair0[g] + npairs[g]; p++) w = std::max(w, last[out_cell[p]] + 1);
        for (long p = pair0[g]; p < pair0[g] + npairs[g]; p++) last[out_cell[p]] = w;
        wave_of[g] = w;
        n_waves = std::max(n_waves, w + 1);
    }
}

template <typename T>
void GemmSet::run_rect(const T* B, T* D, int m, int k, int lda, int nrhs, int trans, int mode,
                       cudaStream_t s, long* launches, bool tables_only)
{
    if (empty()) return;
    const bool waves = mode == GEMM_WAVES;
    if (waves && wave_of.empty()) build_waves();
    auto it = tiles.find(nrhs);
    if (it == tiles.end()) {
        // tiles ordered by wave (a single wave when waves are not used)
        std::vector<int> tg, tc, start;
        const int nw = wave_of.empty() ? 1 : n_waves;
        for (int w = 0; w < nw; w++) {
            start.push_back((int)tg.size());
            for (size_t g = 0; g < npairs.size(); g++) {
                if (!wave_of.empty() && wave_of[g] != w) continue;
                int ncols = npairs[g] * nrhs;
                for (int c = 0; c < ncols; c += GM_BN) {
                    tg.push_back((int)g);
                    tc.push_back(c);
                }
            }
        }
        start.push_back((int)tg.size());
        auto& e = tiles[nrhs];
        e.first.upload(tg);
        e.second.upload(tc);
        wave_tile_start[nrhs] = start;
        it = tiles.find(nrhs);
    }
    if (tables_only) return;
    GemmArgs<T> a;
    a.A = reinterpret_cast<const T* const*>(d_A.p);
    a.g_pair0 = d_pair0.p;
    a.g_npairs = d_npairs.p;
    a.tile_group = it->second.first.p;
    a.tile_col0 = it->second.second.p;
    a.in_cell = d_in.p;
    a.out_cell = d_out.p;
    a.B = B;
    a.D = D;
    a.m = m;
    a.k = k;
    a.lda = lda;
    a.nrhs = nrhs;
    a.trans = trans;
    a.mode = waves ? GEMM_ADD : mode;
    const std::vector<int>& st = wave_tile_start[nrhs];
    const int nw = (int)st.size() - 1;
    if (!waves && nw != 1) throw Error(TBEM_ERR_STATE, "a wave-ordered GEMM set run without waves");
    int dev = 0, sms = 0;
    TBEM_CK(cudaGetDevice(&dev));
    TBEM_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    for (int w = 0; w < nw; w++) {
        const int nt = st[w + 1] - st[w];
        if (nt == 0) continue;
        a.tile_group = it->second.first.p + st[w];
        a.tile_col0 = it->second.second.p + st[w];
        const int bm = gemm_bm(m);
        const long ctas = (long)nt * ((m + bm - 1) / bm);
        // split K when the tiles fill less than two CTAs per SM and the
        // accumulation is atomic anyway (never for the deterministic modes)
        a.kchunk = k;
        int split = 1;
        if (mode == GEMM_ATOMIC && ctas < 2L * sms && k >= 128) {
            const int bk = GemmK<T>::BK;
            split = (int)std::min<long>(std::min<long>((2L * sms + ctas - 1) / ctas, 8), k / 64);
            a.kchunk = ((k + split - 1) / split + bk - 1) / bk * bk;
            split = (k + a.kchunk - 1) / a.kchunk;
        }
        dim3 grid((unsigned)nt, (unsigned)((m + bm - 1) / bm), (unsigned)split);
        if (bm == 128) grouped_gemm_kernel<T, 128><<<grid, GM_THREADS, 0, s>>>(a);
        else grouped_gemm_kernel<T, 64><<<grid, GM_THREADS, 0, s>>>(a);
        TBEM_CK(cudaGetLastError());
        if (launches) (*launches)++;
    }
}

template void GemmSet::run_rect<double>(const double*, double*, int, int, int, int, int, int, cudaStream_t, long*, bool);
template void GemmSet::run_rect<float>(const float*, float*, int, int, int, int, int, int, cudaStream_t, long*, bool);


namespace {
// D[tgt][:] += the target's slots, summed in slot order; one CTA per target,
// the threads over the target's rhs x m values (contiguous in every slot)
__global__ void slot_reduce_kernel(const double* slots, const int* tgt, const int* ptr,
                                   const int* idx, int m, int nrhs, double* D)
{
    const int t = blockIdx.x;
    const long len = (long)nrhs * m;
    const int b = ptr[t], e = ptr[t + 1];
    double* d = D + (long)tgt[t] * len;
    for (long j = threadIdx.x; j < len; j += blockDim.x) {
        double acc = 0.0;
        for (int q = b; q < e; q++) acc += slots[(long)idx[q] * len + j];
        d[j] += acc;
    }
}
}  // namespace

void SlotPlan::build(const GemmSet& G, long cap, const void* pool, size_t esz)
{
    chunks.clear();
    max_slots = 0;
    cap = std::max<long>(cap, 1);
    std::vector<std::pair<int, int>> out_slot;  // (output cell, local slot) of the chunk
    auto close = [&]() {
        if (chunks.empty() || out_slot.empty()) return;
        Chunk& c = chunks.back();
        std::stable_sort(out_slot.begin(), out_slot.end());
        std::vector<int> tgt, ptr{0}, idx;
        for (size_t i = 0; i < out_slot.size(); i++) {
            if (i == 0 || out_slot[i].first != out_slot[i - 1].first) {
                if (i > 0) ptr.push_back((int)idx.size());
                tgt.push_back(out_slot[i].first);
            }
            idx.push_back(out_slot[i].second);
        }
        ptr.push_back((int)idx.size());
        c.tgt.upload(tgt);
        c.ptr.upload(ptr);
        c.idx.upload(idx);
        c.n_tgt = (int)tgt.size();
        c.gemm.upload(pool, esz);
        max_slots = std::max(max_slots, (long)idx.size());
        out_slot.clear();
    };
    long used = cap;  // slots of the open chunk (none open yet)
    for (size_t g = 0; g < G.npairs.size(); g++) {
        long p = G.pair0[g];
        const long p1 = p + G.npairs[g];
        while (p < p1) {
            if (used >= cap) {
                close();
                chunks.emplace_back();
                used = 0;
            }
            const long take = std::min(p1 - p, cap - used);
            std::vector<std::pair<int, int>> pr;
            for (long q = p; q < p + take; q++) {
                pr.push_back({G.in_cell[q], (int)used});
                out_slot.push_back({G.out_cell[q], (int)used});
                used++;
            }
            chunks.back().gemm.add_group(G.A_off[g], pr);
            p += take;
        }
    }
    close();
}

void SlotPlan::run(const double* B, double* D, int m, int nrhs, int trans, double* slots, cudaStream_t s,
                   long* launches)
{
    for (Chunk& c : chunks) {
        c.gemm.run_rect<double>(B, slots, m, m, m, nrhs, trans, GEMM_STORE, s, launches);
        if (c.n_tgt > 0) {
            slot_reduce_kernel<<<c.n_tgt, 256, 0, s>>>(slots, c.tgt.p, c.ptr.p, c.idx.p, m, nrhs, D);
            TBEM_CK(cudaGetLastError());
            if (launches) (*launches)++;
        }
    }
}

// ------------------------------------------------------------ device kernels

namespace {

// Surface point r * (rref * u) + c with the reference's rounding (no FMA),
// TranslationSurface::scale then ::move, cpp/fmm.h:19-40.
__device__ __forceinline__ double surf_coord(double r, double rref, double u, double c)
{
    return __dadd_rn(__dmul_rn(r, __dmul_rn(rref, u)), c);
}

struct SurfJob {
    double tc[3];
    double tr, trref;
    double sc[3];
    double sr, srref;
    long out_off;
};

// Kernel matrix between two translation surfaces, the nbody_matrix layout
// (cpp/nbody_operator.h:87-115): row d1 * ns + i, column d2 * ns + j, weight 1.
__global__ void surf_matrix_kernel(const SurfJob* jobs, const double* unit, int ns, int kid,
                                   KParams kp, double* out)
{
    const SurfJob J = jobs[blockIdx.y];
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)ns * ns) return;
    const int i = (int)(idx / ns), j = (int)(idx % ns);
    const int R = kernel_dim(kid);
    const double ux = unit[3 * i], uy = unit[3 * i + 1], uz = unit[3 * i + 2];
    const double vx = unit[3 * j], vy = unit[3 * j + 1], vz = unit[3 * j + 2];
    const double tx = surf_coord(J.tr, J.trref, ux, J.tc[0]);
    const double ty = surf_coord(J.tr, J.trref, uy, J.tc[1]);
    const double tz = surf_coord(J.tr, J.trref, uz, J.tc[2]);
    const double sx = surf_coord(J.sr, J.srref, vx, J.sc[0]);
    const double sy = surf_coord(J.sr, J.srref, vy, J.sc[1]);
    const double sz = surf_coord(J.sr, J.srref, vz, J.sc[2]);
    double k[9];
    kernel_tensor_any<double>(kid, sx - tx, sy - ty, sz - tz, ux, uy, uz, vx, vy, vz, kp, k);
    const long ld = (long)R * ns;
    double* o = out + J.out_off;
    for (int d1 = 0; d1 < R; d1++)
        for (int d2 = 0; d2 < R; d2++) o[((long)d1 * ns + i) * ld + (long)d2 * ns + j] = k[d1 * R + d2];
}

// Kernel matrix from a leaf's points to a cell surface: row (i * R + d1),
// column d2 * ns + j (the per-leaf L2P operator of the precision form).
__global__ void pts_surf_matrix_kernel(const long* pt0, const int* npts, const int* cell,
                                       const long* row0, const double* xyz, const double* nrm,
                                       const double* center, const double* rad, double rref,
                                       const double* unit, int ns, int kid, KParams kp,
                                       double* out, long out_row_base)
{
    const int t = blockIdx.y;
    const int np = npts[t];
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)np * ns) return;
    const int i = (int)(idx / ns), j = (int)(idx % ns);
    const int R = kernel_dim(kid);
    const long p = pt0[t] + i;
    const int c = cell[t];
    const double vx = unit[3 * j], vy = unit[3 * j + 1], vz = unit[3 * j + 2];
    const double sx = surf_coord(rad[c], rref, vx, center[3 * c]);
    const double sy = surf_coord(rad[c], rref, vy, center[3 * c + 1]);
    const double sz = surf_coord(rad[c], rref, vz, center[3 * c + 2]);
    double k[9];
    kernel_tensor_any<double>(kid, sx - xyz[3 * p], sy - xyz[3 * p + 1], sz - xyz[3 * p + 2],
                          nrm[3 * p], nrm[3 * p + 1], nrm[3 * p + 2], vx, vy, vz, kp, k);
    const long ld = (long)R * ns;
    double* o = out + (row0[t] - out_row_base) * ld;
    for (int d1 = 0; d1 < R; d1++)
        for (int d2 = 0; d2 < R; d2++) o[((long)i * R + d1) * ld + (long)d2 * ns + j] = k[d1 * R + d2];
}

// out = s * in (n values): a level's check-to-equivalent operator from
// another level's, for a kernel homogeneous in the separation
__global__ void scale_copy_kernel(const double* in, double* out, long n, double s)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
        out[t] = s * in[t];
}

// Column k of U (column-major) times 1/s_k, or zero below the cutoff
// (svd_pseudoinverse, cpp/blas_wrapper.cpp:96-127).
__global__ void pinv_scale_kernel(double* U, const double* S, int N, double threshold)
{
    const int k = blockIdx.x;
    const double cutoff = threshold * S[0];
    const double f = S[k] > cutoff ? 1.0 / S[k] : 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) U[(long)k * N + i] *= f;
}

template <typename T>
__global__ void convert_kernel(const double* in, T* out, long n)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = T(in[i]);
}

// s[r][d][i] = w[i] x[r][d][perm[i]]   (tree order; w may be null)
template <typename T>
__global__ void gather_kernel(const double* x, const long* perm, const double* w, T* s, long N,
                              int C, int nrhs)
{
    const long total = N * C * nrhs;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x) {
        const long i = t % N, rd = t / N;
        const double v = x[rd * N + perm[i]];
        s[t] = T(w ? w[i] * v : v);
    }
}

// y[r][d][perm[i]] = w[i] acc[r][d][i]   (w may be null)
__global__ void scatter_kernel(const double* acc, const long* perm, const double* w, double* y,
                               long N, int R, int nrhs)
{
    const long total = N * R * nrhs;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x) {
        const long i = t % N, rd = t / N;
        y[rd * N + perm[i]] = w ? w[i] * acc[t] : acc[t];
    }
}

// rows of length n -> rows of stride ld (the padding columns are zeroed)
template <typename T>
__global__ void convert_rows_kernel(const double* in, T* out, long rows, int n, int ld)
{
    const long total = rows * ld;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x) {
        const long r = t / ld;
        const int k = (int)(t % ld);
        out[t] = k < n ? T(in[r * n + k]) : T(0);
    }
}

// the last r columns (largest eigenvalues) of a column-major n x n
// eigenvector matrix, times scale -> row-major n x r FP32
template <typename T>
__global__ void basis_rows_kernel(const double* evec, int n, int r, double scale, T* out)
{
    const long total = (long)n * r;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x) {
        const long i = t / r;
        const int j = (int)(t % r);
        out[t] = T(scale * evec[(long)(n - r + j) * n + i]);
    }
}

// out[k] = in[k]^T for kb row-major n x n blocks: the column-major view of
// each output block is the row-major matrix itself
__global__ void transpose_blocks_kernel(const double* in, double* out, int n, long kb)
{
    const long nn = (long)n * n, total = kb * nn;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const long k = t / nn, r = t % nn;
        const long j = r / n, i = r % n;
        out[t] = in[k * nn + i * n + j];
    }
}

__global__ void add_kernel(const double* in, float* out, long n)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] += float(in[i]);
}

__global__ void promote_kernel(const float* in, double* out, long n)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = double(in[i]);
}

// Precision-form L2P for many right-hand sides: the same sum with E read
// once per block of L2P_NRB right-hand sides.  One CTA of 64 threads per
// leaf; the block's coefficients sit in shared memory k-major ([ld][NRB],
// every read a broadcast); each thread owns one row of E, streams it with
// float4 loads (the 32 rows of a warp share their cache lines over
// consecutive k) and keeps NRB accumulators.
constexpr int L2P_NRB = 16;
constexpr int L2P_MULTI_THREADS = 64;
template <typename T>
__global__ void __launch_bounds__(L2P_MULTI_THREADS) l2p_multi_kernel(
    const T* E, const long* row0, const int* leaf, const long* pt0, const int* npts, const T* cd,
    int n, int ld, int R, int nrhs, double* y, long y_n)
{
    extern __shared__ __align__(16) unsigned char l2p_smem[];
    T* c = reinterpret_cast<T*>(l2p_smem);  // [ld][L2P_NRB]
    const int t = blockIdx.x;
    const int rows = npts[t] * R;
    const T* c0 = cd + (long)leaf[t] * nrhs * n;
    const T* Et = E + row0[t] * (long)ld;
    for (int r0 = 0; r0 < nrhs; r0 += L2P_NRB) {
        const int nr = min(L2P_NRB, nrhs - r0);
        __syncthreads();
        for (int k = threadIdx.x; k < ld * L2P_NRB; k += blockDim.x) {
            const int kk = k / L2P_NRB, rr = k % L2P_NRB;
            c[k] = (rr < nr && kk < n) ? c0[(long)(r0 + rr) * n + kk] : T(0);
        }
        __syncthreads();
        for (int row = threadIdx.x; row < rows; row += blockDim.x) {
            T acc[L2P_NRB];
#pragma unroll
            for (int q = 0; q < L2P_NRB; q++) acc[q] = T(0);
            const T* er = Et + (long)row * ld;
            for (int k = 0; k < ld; k += 4) {
                T a[4];
                if constexpr (sizeof(T) == 4) {
                    const float4 v = __ldcs(reinterpret_cast<const float4*>(er + k));
                    a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w;
                } else {
                    const double2 v0 = __ldcs(reinterpret_cast<const double2*>(er + k));
                    const double2 v1 = __ldcs(reinterpret_cast<const double2*>(er + k + 2));
                    a[0] = v0.x; a[1] = v0.y; a[2] = v1.x; a[3] = v1.y;
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const T* cb = c + (k + j) * L2P_NRB;
#pragma unroll
                    for (int q = 0; q < L2P_NRB; q++) acc[q] += a[j] * cb[q];
                }
            }
            const int i = row / R, d = row % R;
            for (int q = 0; q < nr; q++) y[((long)(r0 + q) * R + d) * y_n + pt0[t] + i] += (double)acc[q];
        }
    }
}

// Precision-form L2P: y[r][d][pt0 + i] += sum_k E[row0 + i R + d][k] cd[leaf][r][k].
// E rows are padded to ld (a multiple of 128 floats, zero beyond n): one CTA
// per leaf stages the leaf's check potentials of one RHS in shared memory,
// and each warp streams whole rows with float4 loads.  HBM-bound on E.
constexpr int L2P_MAX_LD = 2048;
__global__ void __launch_bounds__(256) l2p_mixed_kernel(const float* E, const long* row0,
                                                        const int* leaf, const long* pt0,
                                                        const int* npts, const float* cd, int n,
                                                        int ld, int R, int nrhs, double* y, long y_n)
{
    __shared__ __align__(16) float c[L2P_MAX_LD];
    const int t = blockIdx.x;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = blockDim.x / 32;
    const int rows = npts[t] * R;
    const float* c0 = cd + (long)leaf[t] * nrhs * n;
    const float4* cv = reinterpret_cast<const float4*>(c);
    for (int r = 0; r < nrhs; r++) {
        __syncthreads();
        for (int k = threadIdx.x; k < ld; k += blockDim.x) c[k] = k < n ? c0[(long)r * n + k] : 0.f;
        __syncthreads();
        // four rows per warp at a time: their loads are in flight together; E
        // is read once per apply, so it streams past L2 (evict-first loads)
        for (int rb = warp * 4; rb < rows; rb += nw * 4) {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            for (int k4 = lane; k4 < ld / 4; k4 += 32) {
                const float4 b = cv[k4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    if (rb + q < rows) {
                        const float4 a = __ldcs(reinterpret_cast<const float4*>(E + (row0[t] + rb + q) * (long)ld) + k4);
                        acc[q] += a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
            if (lane < 4 && rb + lane < rows) {
                const int row = rb + lane;
                const float v = lane == 0 ? acc[0] : lane == 1 ? acc[1] : lane == 2 ? acc[2] : acc[3];
                const int i = row / R, d = row % R;
                y[((long)r * R + d) * y_n + pt0[t] + i] += (double)v;
            }
        }
    }
}

// Its transpose: cd[leaf][r][k] = sum_rows E[row][k] z[r][d][pt0 + i].
template <typename T>
__global__ void l2p_mixed_t_kernel(const T* E, const long* row0, const int* leaf,
                                   const long* pt0, const int* npts, const T* z, long z_n,
                                   int n, int ld, int R, int nrhs, T* cd)
{
    const int t = blockIdx.x;
    const int rows = npts[t] * R;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        for (int r = 0; r < nrhs; r++) {
            T acc = 0;
            for (int row = 0; row < rows; row++) {
                const int i = row / R, d = row % R;
                acc += E[(row0[t] + row) * (long)ld + k] * z[((long)r * R + d) * z_n + pt0[t] + i];
            }
            cd[((long)leaf[t] * nrhs + r) * n + k] = acc;
        }
    }
}

inline unsigned grid_for(long n, int threads = 256)
{
    long b = (n + threads - 1) / threads;
    return (unsigned)std::max<long>(1, std::min<long>(b, 152L * 64));
}

inline double hypot_ref(const double* v)
{
    return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
}

}  // namespace

// Homogeneity degree of a 3D kernel in the separation (K(s d) = s^deg K(d)
// for s > 0); 1 (not homogeneous) for the 2D kernels, whose logarithms are not.
namespace {
int kernel_degree(int kid)
{
    switch (kid) {
    case LAP_S: case EL_DISP: return -1;
    case LAP_D: case EL_TRAC: case EL_ADJ: return -2;
    case EL_HYP: return -3;
    case IDENT: return 0;
    default: return 1;
    }
}
}  // namespace

// ------------------------------------------------------------------ plan

Plan::~Plan()
{
    // the library handles are released on the device they were made on
    int prev = -1;
    const bool own = !opt.host_only && cudaGetDevice(&prev) == cudaSuccess && prev != opt.device &&
                     cudaSetDevice(opt.device) == cudaSuccess;
    cudaGetLastError();
    for (auto& m : marks) cudaEventDestroy(m.second);
    for (auto e : event_pool) cudaEventDestroy(e);
    if (h_err) cudaFreeHost(h_err);
    if (cublas) cublasDestroy(cublas);
    if (solver) cusolverDnDestroy(solver);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
    if (own) cudaSetDevice(prev);
}

void Plan::upload_tree(const Tree& t, const double* locs, const double* normals,
                       const double* weights, DTree& d)
{
    const long N = t.n_points();
    std::vector<double> xyz(3 * N), nrm(3 * N), w;
    std::vector<float> nrm32(3 * N);
    for (long i = 0; i < N; i++) {
        long o = t.perm[i];
        for (int k = 0; k < 3; k++) {
            xyz[3 * i + k] = locs[3 * o + k];
            nrm[3 * i + k] = normals[3 * o + k];
            nrm32[3 * i + k] = (float)normals[3 * o + k];
        }
    }
    if (weights) {
        w.resize(N);
        for (long i = 0; i < N; i++) w[i] = weights[t.perm[i]];
        d.w.upload(w);
    }
    d.xyz.upload(xyz);
    d.nrm64.upload(nrm);
    d.nrm32.upload(nrm32);
    d.perm.upload(t.perm);
    std::vector<double> c(3 * t.cells.size()), r(t.cells.size());
    for (size_t i = 0; i < t.cells.size(); i++) {
        for (int k = 0; k < 3; k++) c[3 * i + k] = t.cells[i].center[k];
        r[i] = hypot_ref(t.cells[i].hw);
    }
    d.center.upload(c);
    d.rad.upload(r);
}

void Plan::build(int kernel, const double* params, const double* obs_locs,
                 const double* obs_normals, long n_obs_, const double* src_locs,
                 const double* src_normals, const double* src_weights, long n_src_,
                 const TbemFmmConfig& cfg_, const TbemGpuOptions& opt_)
{
    if (!kernel_valid(kernel)) throw Error(TBEM_ERR_ARG, "unknown kernel id");
    if (cfg_.min_pts_per_cell <= 0) throw Error(TBEM_ERR_ARG, "min_pts_per_cell must be > 0");
    if (cfg_.order <= 0) throw Error(TBEM_ERR_ARG, "order must be > 0");
    if (!(cfg_.mac > 0)) throw Error(TBEM_ERR_ARG, "mac must be > 0");
    if (n_obs_ < 0 || n_src_ < 0) throw Error(TBEM_ERR_ARG, "negative point count");
    if ((n_obs_ > 0 && (!obs_locs || !obs_normals)) ||
        (n_src_ > 0 && (!src_locs || !src_normals || !src_weights)))
        throw Error(TBEM_ERR_ARG, "null point array");
    if (opt_.precision < TBEM_PRECISION_FP64 || opt_.precision > TBEM_PRECISION_FP64_COMPRESSED)
        throw Error(TBEM_ERR_ARG, "unknown precision form");
    setup_start();
    kid = kernel;
    R = kernel_dim(kid);
    sdim = kernel_space_dim(kid);
    if (sdim == 2 && opt_.precision != TBEM_PRECISION_FP64)
        throw Error(TBEM_ERR_ARG, "2D kernels run in the plain FP64 form only (the precision "
                                  "form's operator reuse needs the 3D kernels' homogeneity)");
    mu = (params && R > 1) ? params[0] : 1.0;
    nu = (params && R > 1) ? params[1] : 0.25;
    kp = make_kparams(kid, mu, nu);
    cfg = cfg_;
    opt = opt_;
    if (!(opt.svd_threshold > 0)) opt.svd_threshold = 1e-10;
    n_obs = n_obs_;
    n_src = n_src_;
    // points are [n][sdim]; kept as [n][3] (z = 0 in 2D)
    auto widen = [&](std::vector<double>& dst, const double* p, long n) {
        dst.assign(3 * n, 0.0);
        for (long i = 0; i < n; i++)
            for (int d = 0; d < sdim; d++) dst[3 * i + d] = p[sdim * i + d];
    };
    widen(h_obs_locs, obs_locs, n_obs);
    widen(h_obs_normals, obs_normals, n_obs);
    widen(h_src_locs, src_locs, n_src);
    widen(h_src_normals, src_normals, n_src);
    h_src_weights.assign(src_weights, src_weights + n_src);

    std::unique_ptr<DeviceGuard> guard;
    if (!opt.host_only) {
        guard.reset(new DeviceGuard(opt.device));
        create_streams();
    }

    same_tree = n_obs == n_src &&
                (n_obs == 0 || std::memcmp(h_obs_locs.data(), h_src_locs.data(),
                                           3 * n_obs * sizeof(double)) == 0);
    // The precision forms with different observation and source points cut
    // both trees from one cube (the bounding cube of all points): the cells
    // of a level are then the same cubes in both trees, every M2L pair is an
    // integer offset between congruent cells, and the M2L operators are
    // precomputed (and compressed) as for a single tree.  The plain form
    // keeps the reference's trees (each over its own bounding box).
    common_cube = !same_tree && sdim == 3 && opt.precision != TBEM_PRECISION_FP64 && n_obs > 0 &&
                  n_src > 0;
    if (common_cube) {
        double mn[3], mx[3];
        for (int d = 0; d < 3; d++) mn[d] = mx[d] = h_obs_locs[d];
        for (const std::vector<double>* v : {&h_obs_locs, &h_src_locs})
            for (size_t i = 0; i < v->size() / 3; i++)
                for (int d = 0; d < 3; d++) {
                    mn[d] = std::min(mn[d], (*v)[3 * i + d]);
                    mx[d] = std::max(mx[d], (*v)[3 * i + d]);
                }
        double c[3], H = 0;
        for (int d = 0; d < 3; d++) {
            c[d] = (mx[d] + mn[d]) / 2.0;
            H = std::max(H, (mx[d] - mn[d]) / 2.0);
        }
        if (!(H > 0)) H = 1.0;
        otree = build_tree_cube(h_obs_locs.data(), n_obs, cfg.min_pts_per_cell, c, H);
        stree_own = build_tree_cube(h_src_locs.data(), n_src, cfg.min_pts_per_cell, c, H);
        stree = &stree_own;
    } else {
        otree = build_tree(h_obs_locs.data(), n_obs, cfg.min_pts_per_cell, sdim);
        if (same_tree) {
            stree = &otree;
        } else {
            stree_own = build_tree(h_src_locs.data(), n_src, cfg.min_pts_per_cell, sdim);
            stree = &stree_own;
        }
    }
    unit = sdim == 2 ? circle_surface(cfg.order) : sphere_surface(cfg.order);
    ns = (int)(unit.size() / 3);
    n = R * ns;
    L = build_lists(otree, *stree, cfg.mac, ns, cfg.account_for_small_cells != 0);
    setup_mark("trees_lists");
    if (opt.host_only) return;
    finish_build(h_obs_locs.data(), h_obs_normals.data(), h_src_locs.data(), h_src_normals.data(),
                 h_src_weights.data());
}

void Plan::create_streams()
{
    TBEM_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    TBEM_CK(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    TBEM_CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    TBEM_CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    TBEM_CKB(cublasCreate(&cublas));
    TBEM_CKB(cublasSetStream(cublas, stream));
    TBEM_CKS(cusolverDnCreate(&solver));
    TBEM_CKS(cusolverDnSetStream(solver, stream));
}

// Device side of a build once the trees and lists exist: the trees' points
// (in the coordinates the operators are built in), the task sets, the
// form's operators and the autotuned launch shapes.
void Plan::finish_build(const double* o_locs, const double* o_nrm, const double* s_locs,
                        const double* s_nrm, const double* s_w)
{
    d_unit.upload(unit);
    upload_tree(otree, o_locs, o_nrm, nullptr, dobs);
    upload_tree(*stree, s_locs, s_nrm, s_w, dsrc_own);
    dsrc = &dsrc_own;
    build_tasks();
    setup_mark("upload_tasks");
    build_form();
    TBEM_CK(cudaStreamSynchronize(stream));
    if (opt.p2p_block == 2 || opt.p2p_block == 4 || opt.p2p_block == 8) p2p_tpt = opt.p2p_block;
    else autotune_p2p();
    if (opt.p2m_block == 1 || opt.p2m_block == 2 || opt.p2m_block == 4) p2m_tpt = opt.p2m_block;
    else autotune_p2m();
    autotune_tc();
    setup_mark("autotune");
}

// The batched form: n_meshes independent point sets (observation = source
// points within each mesh) in one plan.  Mesh m is moved and scaled into the
// cube [-1, 1]^3 (x' = (x - c_m) / H_m, c_m its bounding box's centre, H_m
// its largest half width) and its tree is cut from that cube, so every
// mesh's level-l cells are the same cubes of half width 2^-l and all meshes
// share one set of check-to-equivalent and translation operators.  The
// kernel is homogeneous of degree deg in the separation at fixed normals,
// K(x, y) = H^deg K(x', y'), so the weights become w' = H^deg w and the
// scaled problem has exactly the original's outputs.  The trees of the
// meshes form one forest (level-major), and the task lists of all meshes
// are concatenated: every pass of an apply covers every mesh in one launch
// per pass (per level for M2M / L2L).
void Plan::build_batch(int kernel, const double* params, int n_meshes, const long* offsets,
                       const double* locs, const double* normals, const double* weights,
                       const TbemFmmConfig& cfg_, const TbemGpuOptions& opt_)
{
    if (!kernel_valid(kernel) || kernel_space_dim(kernel) != 3)
        throw Error(TBEM_ERR_ARG, "the batched form takes the 3D kernel ids 0..6");
    if (cfg_.min_pts_per_cell <= 0) throw Error(TBEM_ERR_ARG, "min_pts_per_cell must be > 0");
    if (cfg_.order <= 0) throw Error(TBEM_ERR_ARG, "order must be > 0");
    if (!(cfg_.mac > 0)) throw Error(TBEM_ERR_ARG, "mac must be > 0");
    if (cfg_.account_for_small_cells)
        throw Error(TBEM_ERR_ARG, "the batched form has no small-cell routing");
    if (opt_.precision < TBEM_PRECISION_FP64 || opt_.precision > TBEM_PRECISION_FP64_COMPRESSED)
        throw Error(TBEM_ERR_ARG, "unknown precision form");
    if (n_meshes < 0 || (n_meshes > 0 && !offsets)) throw Error(TBEM_ERR_ARG, "bad mesh offsets");
    if (n_meshes > 0 && offsets[0] != 0) throw Error(TBEM_ERR_ARG, "mesh offsets must start at 0");
    for (int m = 0; m < n_meshes; m++)
        if (offsets[m + 1] < offsets[m]) throw Error(TBEM_ERR_ARG, "mesh offsets must not decrease");
    const long N = n_meshes > 0 ? offsets[n_meshes] : 0;
    if (N > 0 && (!locs || !normals || !weights)) throw Error(TBEM_ERR_ARG, "null point array");
    setup_start();
    kid = kernel;
    R = kernel_dim(kid);
    sdim = 3;
    mu = (params && R > 1) ? params[0] : 1.0;
    nu = (params && R > 1) ? params[1] : 0.25;
    kp = make_kparams(kid, mu, nu);
    cfg = cfg_;
    opt = opt_;
    if (!(opt.svd_threshold > 0)) opt.svd_threshold = 1e-10;
    n_obs = n_src = N;
    batch_off.assign(offsets, offsets + n_meshes + 1);
    h_obs_locs.assign(locs, locs + 3 * N);
    h_obs_normals.assign(normals, normals + 3 * N);
    h_src_locs = h_obs_locs;
    h_src_normals = h_obs_normals;
    h_src_weights.assign(weights, weights + N);

    const int deg = kernel_degree(kid);
    std::vector<double> xl(3 * N), xw(N);
    batch_center.assign(3 * (size_t)n_meshes, 0.0);
    batch_scale.assign(n_meshes, 1.0);
    std::vector<Tree> trees(n_meshes);
    std::vector<TaskLists> lists(n_meshes);
    unit = sphere_surface(cfg.order);
    ns = (int)(unit.size() / 3);
    n = R * ns;
    const double origin[3] = {0.0, 0.0, 0.0};
    nf::parallel_for(
        n_meshes,
        [&](long m) {
            const long p0 = offsets[m], p1 = offsets[m + 1];
            double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
            for (long i = p0; i < p1; i++)
                for (int d = 0; d < 3; d++) {
                    const double v = locs[3 * i + d];
                    if (i == p0 || v < mn[d]) mn[d] = v;
                    if (i == p0 || v > mx[d]) mx[d] = v;
                }
            double c[3], H = 0;
            for (int d = 0; d < 3; d++) {
                c[d] = (mx[d] + mn[d]) / 2.0;
                H = std::max(H, (mx[d] - mn[d]) / 2.0);
            }
            if (!(H > 0)) H = 1.0;  // a single point (or coincident points)
            for (int d = 0; d < 3; d++) batch_center[3 * m + d] = c[d];
            batch_scale[m] = H;
            const double wscale = std::pow(H, (double)deg);
            for (long i = p0; i < p1; i++) {
                for (int d = 0; d < 3; d++) xl[3 * i + d] = (locs[3 * i + d] - c[d]) / H;
                xw[i] = weights[i] * wscale;
            }
            trees[m] = build_tree_cube(&xl[3 * p0], p1 - p0, cfg.min_pts_per_cell, origin, 1.0);
            lists[m] = build_lists(trees[m], trees[m], cfg.mac, ns, false);
        },
        1);
    std::vector<std::vector<int>> gid;
    otree = merge_forest(trees, std::vector<long>(offsets, offsets + std::max(n_meshes, 0)), gid);
    trees.clear();
    L = merge_lists(lists, gid);
    lists.clear();
    same_tree = true;
    stree = &otree;
    setup_mark("trees_lists");
    if (opt.host_only) return;
    DeviceGuard guard(opt.device);
    create_streams();
    finish_build(xl.data(), h_obs_normals.data(), xl.data(), h_obs_normals.data(), xw.data());
}

// Picks the tensor-core GEMM's N tile for the M2L set (and uses it for the
// level translations too) by timing both shapes on this operator's own pair
// lists with zero operands (the cost does not depend on the values).
void Plan::autotune_tc()
{
    const bool comp = f.use_tc_c && !f.m2l_c.empty();
    if (!comp && (!f.use_tc || f.m2l.empty())) return;
    ensure_rhs(1);
    const long ncs = (long)stree->cells.size(), nco = (long)otree.cells.size();
    TcPlanes& P = comp ? f.tc_c : f.tc;
    GemmSet& G = comp ? f.m2l_c : f.m2l;
    float* in = comp ? cuc32.p : cu32.p;
    float* out = comp ? cdc32.p : cd32.p;
    const long nn = comp ? (long)f.r_out * f.r_in : (long)n * n;
    TBEM_CK(cudaMemsetAsync(in, 0, sizeof(float) * ncs * P.k, stream));
    P.split_b_rows(in, 0, ncs, std::max(ncs, nco), stream);
    ScopedEvent t0, t1;
    const cudaEvent_t e0 = t0.e, e1 = t1.e;
    // every timed run starts from a cold L2 (a 256 MB write evicts it), as
    // the M2L of an apply does: with the operator planes left in L2 between
    // runs the 32-deep shape looked fastest, cold it was 25 % slower
    DBuf<char> flush;
    constexpr size_t FLUSH_BYTES = 256u << 20;
    flush.alloc(FLUSH_BYTES);
    float best = 1e30f;
    int best_bn = 128, best_bk = 64;
    const int shapes[4][2] = {{128, 64}, {64, 64}, {128, 32}, {256, 32}};
    const int fixed = opt.tc_shape >= 1 && opt.tc_shape <= 4 ? opt.tc_shape - 1 : -1;
    for (int si = 0; si < 4; si++) {
        const auto& sh = shapes[si];
        if (fixed >= 0 && si != fixed) continue;
        G.tc_bn = sh[0];
        G.tc_bk = sh[1];
        float ms = 1e30f;  // best of five (the first also builds the tile tables)
        for (int rep = 0; rep < 6; rep++) {
            TBEM_CK(cudaMemsetAsync(flush.p, rep, FLUSH_BYTES, stream));
            TBEM_CK(cudaEventRecord(e0, stream));
            G.run_tc(P, out, 1, 1, nn, stream, nullptr);
            TBEM_CK(cudaEventRecord(e1, stream));
            TBEM_CK(cudaEventSynchronize(e1));
            float t = 0.f;
            TBEM_CK(cudaEventElapsedTime(&t, e0, e1));
            if (rep > 0) ms = std::min(ms, t);
        }
        if (ms < best) {
            best = ms;
            best_bn = sh[0];
            best_bk = sh[1];
        }
    }
    G.tc_bn = best_bn;
    G.tc_bk = best_bk;
    for (auto& g : f.m2m) { g.tc_bn = best_bn; g.tc_bk = best_bk; }
    for (auto& g : f.l2l) { g.tc_bn = best_bn; g.tc_bk = best_bk; }
}

// Picks the point-to-point pass's threads per target (2, 4 or 8) by timing
// each variant on this operator's own task lists (zero densities: the cost
// does not depend on the values).
void Plan::autotune_p2p()
{
    if (p2p.n_items() == 0) return;
    ensure_rhs(1);
    const bool mixed = f.mixed && !f.f64;  // FP32 evaluation passes
    if (mixed) TBEM_CK(cudaMemsetAsync(s32.p, 0, sizeof(float) * R * n_src, stream));
    else TBEM_CK(cudaMemsetAsync(s64.p, 0, sizeof(double) * R * n_src, stream));
    ScopedEvent t0, t1;
    const cudaEvent_t e0 = t0.e, e1 = t1.e;
    float best = 1e30f;
    int best_tpt = 4;
    for (int tpt : {4, 2, 8}) {
        p2p_tpt = tpt;
        float ms = 0.f;
        for (int rep = 0; rep < 3; rep++) {
            TBEM_CK(cudaEventRecord(e0, stream));
            if (mixed)
                eval<float>(p2p_set(), kid, false, false, otree, dobs, 0, *dsrc, 0, s32.p, n_src,
                            nullptr, y64.p, n_obs, nullptr, 1, 1, stream, false);
            else
                eval<double>(p2p_set(), kid, false, false, otree, dobs, 0, *dsrc, 0, s64.p, n_src,
                             nullptr, y64.p, n_obs, nullptr, 1, 1, stream, false);
            TBEM_CK(cudaEventRecord(e1, stream));
            TBEM_CK(cudaEventSynchronize(e1));
            float t = 0.f;
            TBEM_CK(cudaEventElapsedTime(&t, e0, e1));
            if (rep > 0) ms += t;  // the first run warms the caches
        }
        if (ms < best) {
            best = ms;
            best_tpt = tpt;
        }
    }
    p2p_tpt = best_tpt;
}

// Picks the points-to-check-surface pass's threads per target (1, 2 or 4)
// the same way: each variant timed on this operator's own leaves.
void Plan::autotune_p2m()
{
    if (p2m.n_items() == 0) return;
    ensure_rhs(1);
    const bool mixed = f.mixed && !f.f64;  // FP32 evaluation passes
    if (mixed) TBEM_CK(cudaMemsetAsync(s32.p, 0, sizeof(float) * R * n_src, stream));
    else TBEM_CK(cudaMemsetAsync(s64.p, 0, sizeof(double) * R * n_src, stream));
    ScopedEvent t0, t1;
    const cudaEvent_t e0 = t0.e, e1 = t1.e;
    float best = 1e30f;
    int best_tpt = 4;
    for (int tpt : {4, 2, 1}) {
        p2m_tpt = tpt;
        float ms = 0.f;
        for (int rep = 0; rep < 3; rep++) {
            TBEM_CK(cudaEventRecord(e0, stream));
            if (mixed)
                eval<float>(p2m_set(), f.ks_kid, true, false, *stree, *dsrc, f.r_uc, *dsrc, 0, s32.p, n_src,
                            nullptr, nullptr, 0, cu32.p, 0, 1, stream, false);
            else
                eval<double>(p2m_set(), f.ks_kid, true, false, *stree, *dsrc, f.r_uc, *dsrc, 0, s64.p, n_src,
                             nullptr, nullptr, 0, cu64.p, 0, 1, stream, false);
            TBEM_CK(cudaEventRecord(e1, stream));
            TBEM_CK(cudaEventSynchronize(e1));
            float t = 0.f;
            TBEM_CK(cudaEventElapsedTime(&t, e0, e1));
            if (rep > 0) ms += t;
        }
        if (ms < best) {
            best = ms;
            best_tpt = tpt;
        }
    }
    p2m_tpt = best_tpt;
}

void Plan::build_tasks()
{
    const Tree& O = otree;
    const Tree& S = *stree;
    constexpr int TPB = EVAL_THREADS / 4;
    // forward
    for (int c : L.p2m) {
        const Cell& cc = S.cells[c];
        p2m.add(c, ns, cc.center, {{cc.pt_begin, (int)cc.n_points()}}, TPB);
        p2m_tpt1.add(c, ns, cc.center, {{cc.pt_begin, (int)cc.n_points()}}, EVAL_THREADS);
        p2m_tpt2.add(c, ns, cc.center, {{cc.pt_begin, (int)cc.n_points()}}, EVAL_THREADS / 2);
    }
    std::vector<std::vector<int>> p2p_of(O.cells.size()), m2p_of(O.cells.size()),
        p2l_of(O.cells.size()), m2l_of(O.cells.size());
    std::vector<std::vector<int>> p2p_by_src(S.cells.size()), m2p_by_src(S.cells.size()),
        p2l_by_src(S.cells.size()), m2l_by_src(S.cells.size());
    for (auto& p : L.p2p) { p2p_of[p.obs].push_back(p.src); p2p_by_src[p.src].push_back(p.obs); }
    for (auto& p : L.m2p) { m2p_of[p.obs].push_back(p.src); m2p_by_src[p.src].push_back(p.obs); }
    for (auto& p : L.p2l) { p2l_of[p.obs].push_back(p.src); p2l_by_src[p.src].push_back(p.obs); }

    // M2L keys: (obs level, src level, integer offset in units of the finer
    // half width), numbered in order of first appearance.  Found first: the
    // on-the-fly M2L task sets below are built only when the pairs are not
    // all integer offsets between congruent cells.
    m2l_groups.clear();
    m2l_key_ls.clear();
    m2l_canon.clear();
    f.m2l_on_the_fly = !(same_tree || common_cube);
    if (same_tree || common_cube) {
        // open-addressing table of packed keys (levels < 256, offsets within
        // +-2^15: beyond that the pair is computed on the fly)
        std::vector<unsigned long long> hkey(1024, ~0ull);
        std::vector<int> hval(1024, -1);
        auto slot_of = [&](unsigned long long k) {
            unsigned long long h = k * 0x9e3779b97f4a7c15ull;
            size_t i = (size_t)(h >> 20) & (hkey.size() - 1);
            while (hkey[i] != ~0ull && hkey[i] != k) i = (i + 1) & (hkey.size() - 1);
            return i;
        };
        for (size_t pi = 0; pi < L.m2l.size() && !f.m2l_on_the_fly; pi++) {
            const Cell& o = O.cells[L.m2l[pi].obs];
            const Cell& sc = S.cells[L.m2l[pi].src];
            const double* hf = o.level >= sc.level ? o.hw : sc.hw;
            long off[3];
            for (int d = 0; d < 3; d++) {
                double delta = sc.center[d] - o.center[d];
                if (hf[d] == 0.0) {
                    if (delta != 0.0) f.m2l_on_the_fly = true;
                    off[d] = 0;
                    continue;
                }
                double q = delta / hf[d];
                double r = std::nearbyint(q);
                if (std::fabs(q - r) > 1e-6 * std::max(1.0, std::fabs(q))) f.m2l_on_the_fly = true;
                if (std::fabs(r) >= 32767.0) f.m2l_on_the_fly = true;
                off[d] = (long)r;
            }
            if (f.m2l_on_the_fly || o.level > 255 || sc.level > 255) {
                f.m2l_on_the_fly = true;
                break;
            }
            const unsigned long long key =
                ((unsigned long long)o.level << 56) | ((unsigned long long)sc.level << 48) |
                ((unsigned long long)(off[0] + 32768) << 32) | ((unsigned long long)(off[1] + 32768) << 16) |
                (unsigned long long)(off[2] + 32768);
            size_t i = slot_of(key);
            int g = hval[i];
            if (g < 0) {
                g = (int)m2l_groups.size();
                hkey[i] = key;
                hval[i] = g;
                m2l_groups.push_back({});
                m2l_key_ls.push_back(sc.level);
                m2l_canon.push_back({L.m2l[pi].obs, L.m2l[pi].src});
                if (2 * m2l_groups.size() > hkey.size()) {  // keep the load under one half
                    std::vector<unsigned long long> ok(hkey.size() * 2, ~0ull);
                    std::vector<int> ov(hkey.size() * 2, -1);
                    ok.swap(hkey);
                    ov.swap(hval);
                    for (size_t j = 0; j < ok.size(); j++)
                        if (ok[j] != ~0ull) {
                            const size_t t = slot_of(ok[j]);
                            hkey[t] = ok[j];
                            hval[t] = ov[j];
                        }
                }
            }
            m2l_groups[g].push_back((int)pi);
        }
        if (f.m2l_on_the_fly) {
            m2l_groups.clear();
            m2l_key_ls.clear();
            m2l_canon.clear();
        }
    }

    // the per-cell M2L lists feed only the on-the-fly M2L task sets
    if (f.m2l_on_the_fly)
        for (auto& p : L.m2l) { m2l_of[p.obs].push_back(p.src); m2l_by_src[p.src].push_back(p.obs); }

    // A source cell "touches" a target leaf when their boxes overlap or share
    // a face, edge or corner: its pairs are the closest ones, where the FP32
    // double layer takes the double-float n . d
    auto touches = [](const Cell& a, const Cell& b) {
        for (int d = 0; d < 3; d++) {
            const double gap = std::fabs(a.center[d] - b.center[d]) - a.hw[d] - b.hw[d];
            if (gap > 1e-9 * std::max(a.hw[d] + b.hw[d], 1e-300)) return false;
        }
        return true;
    };
    // point targets collect the lists of the leaf and of all its ancestors
    for (size_t c = 0; c < O.cells.size(); c++) {
        const Cell& leaf = O.cells[c];
        if (!leaf.is_leaf()) continue;
        std::vector<std::pair<long, int>> pp, mp;
        std::vector<int> near;
        for (int a = (int)c; a >= 0; a = O.cells[a].parent) {
            for (int s : p2p_of[a]) {
                pp.push_back({S.cells[s].pt_begin, (int)S.cells[s].n_points()});
                near.push_back(touches(leaf, S.cells[s]) ? 1 : 0);
            }
            for (int s : m2p_of[a]) mp.push_back({s, ns});
        }
        p2p.add(leaf.pt_begin, (int)leaf.n_points(), leaf.center, pp, TPB, near);
        p2p_tpt2.add(leaf.pt_begin, (int)leaf.n_points(), leaf.center, pp, EVAL_THREADS / 2, near);
        p2p_tpt8.add(leaf.pt_begin, (int)leaf.n_points(), leaf.center, pp, EVAL_THREADS / 8, near);
        m2p.add(leaf.pt_begin, (int)leaf.n_points(), leaf.center, mp, TPB);
    }
    for (size_t c = 0; c < O.cells.size(); c++) {
        const Cell& oc = O.cells[c];
        std::vector<std::pair<long, int>> pl, ml;
        for (int s : p2l_of[c]) pl.push_back({S.cells[s].pt_begin, (int)S.cells[s].n_points()});
        for (int s : m2l_of[c]) ml.push_back({s, ns});
        p2l.add((long)c, ns, oc.center, pl, TPB);
        if (f.m2l_on_the_fly) m2l_fly.add((long)c, ns, oc.center, ml, TPB);
    }
    for (int c : L.l2p) {
        const Cell& cc = O.cells[c];
        l2p.add(cc.pt_begin, (int)cc.n_points(), cc.center, {{c, ns}}, TPB);
    }
    // transposed: targets live in the source tree, sources in the observation tree
    for (int c : L.p2m) {
        const Cell& cc = S.cells[c];
        p2m_t.add(cc.pt_begin, (int)cc.n_points(), cc.center, {{c, ns}}, TPB);
    }
    for (size_t c = 0; c < S.cells.size(); c++) {
        const Cell& leaf = S.cells[c];
        if (!leaf.is_leaf()) continue;
        std::vector<std::pair<long, int>> pp, pl;
        for (int a = (int)c; a >= 0; a = S.cells[a].parent) {
            for (int o : p2p_by_src[a]) pp.push_back({O.cells[o].pt_begin, (int)O.cells[o].n_points()});
            for (int o : p2l_by_src[a]) pl.push_back({o, ns});
        }
        p2p_t.add(leaf.pt_begin, (int)leaf.n_points(), leaf.center, pp, TPB);
        p2l_t.add(leaf.pt_begin, (int)leaf.n_points(), leaf.center, pl, TPB);
    }
    for (size_t c = 0; c < S.cells.size(); c++) {
        const Cell& sc = S.cells[c];
        std::vector<std::pair<long, int>> mp, ml;
        for (int o : m2p_by_src[c]) mp.push_back({O.cells[o].pt_begin, (int)O.cells[o].n_points()});
        for (int o : m2l_by_src[c]) ml.push_back({o, ns});
        m2p_t.add((long)c, ns, sc.center, mp, TPB);
        if (f.m2l_on_the_fly) m2l_fly_t.add((long)c, ns, sc.center, ml, TPB);
    }
    for (int c : L.l2p) {
        const Cell& cc = O.cells[c];
        l2p_t.add(c, ns, cc.center, {{cc.pt_begin, (int)cc.n_points()}}, TPB);
    }
    p2p_tpt2.tpt = 2;
    p2p_tpt8.tpt = 8;
    p2m_tpt1.tpt = 1;
    p2m_tpt2.tpt = 2;
    for (TaskSet* t : {&p2m, &p2m_tpt1, &p2m_tpt2, &p2p, &p2p_tpt2, &p2p_tpt8, &m2p, &p2l, &l2p, &m2l_fly, &p2m_t, &p2p_t,
                       &m2p_t, &p2l_t, &l2p_t, &m2l_fly_t})
        t->upload();

    // dedup keys of the M2M / L2L octant translations and the M2L translations
    const int LS = S.n_levels(), LO = O.n_levels();
    m2m_pairs.assign(std::max(LS, 1) * 8, {});
    m2m_canon.assign(std::max(LS, 1) * 8, {-1, -1});
    for (int c : L.m2m) {
        const Cell& p = S.cells[c];
        for (int k = 0; k < p.n_children; k++) {
            int ch = p.first_child + k;
            int key = p.level * 8 + S.cells[ch].octant;
            if (m2m_canon[key].first < 0) m2m_canon[key] = {c, ch};
            m2m_pairs[key].push_back({ch, c});  // (in = child, out = parent)
        }
    }
    l2l_pairs.assign(std::max(LO, 1) * 8, {});
    l2l_canon.assign(std::max(LO, 1) * 8, {-1, -1});
    for (int c : L.l2l) {
        const Cell& p = O.cells[c];
        for (int k = 0; k < p.n_children; k++) {
            int ch = p.first_child + k;
            int key = p.level * 8 + O.cells[ch].octant;
            if (l2l_canon[key].first < 0) l2l_canon[key] = {c, ch};
            l2l_pairs[key].push_back({c, ch});  // (in = parent, out = child)
        }
    }
}

// Pseudo-inverses of the check-to-equivalent systems of every level
// (build_check_to_equiv + svd_inverse_nbody, cpp/fmm.cpp:113-160), FP64 on
// the GPU with cuSOLVER gesvd.  Every level's system is the same pair of
// concentric spheres scaled by the level's cell radius r_l, so for a 3D
// kernel homogeneous of degree deg the system of level l is (r_l / r_0)^deg
// times that of level 0 and its pseudo-inverse (the same relative cutoff) is
// (r_l / r_0)^-deg times level 0's: one SVD per tree side.  Levels whose
// sphere separation falls below 1e-5 (where the r^2 < 1e-12 self-pair rule
// could drop entries) and the 2D kernels get their own SVD, as in the
// reference.  The scaled operators differ from per-level SVDs by rounding of
// the size of the reference's own one-ulp sensitivity.
namespace {
// Pseudo-inverses factored in this process, by everything the factored
// system depends on (kernel and its parameters, the unit surface, the
// surface radii and centre, the cut-off, the device).  Operators that share
// a translation kernel over the same tree -- the displacement and traction
// operators of one mesh, or a clone -- then factor each level once.  The
// values are host copies (n^2 doubles each), the oldest dropped past
// C2E_CACHE_BYTES.
using C2EKey = std::tuple<int, int, int, double, double, double, double, double, double, double,
                          double, double, uint64_t, int>;
constexpr size_t C2E_CACHE_BYTES = 512u << 20;
std::mutex c2e_cache_mu;
std::map<C2EKey, std::vector<double>> c2e_cache;
std::vector<C2EKey> c2e_cache_order;
size_t c2e_cache_bytes = 0;

// FNV-1a over bytes, from a given basis (two bases give two hashes)
uint64_t hash_bytes(const void* p, size_t n, uint64_t h = 1469598103934665603ull)
{
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

uint64_t hash_doubles(const std::vector<double>& v)
{
    return hash_bytes(v.data(), v.size() * sizeof(double));
}

// The eigen-decompositions of the M2L Gram matrices (both n x n eigenvector
// sets and their 2n eigenvalues), by two hashes of the M2L matrices'
// description (kernel, parameters, unit surface, every class's surfaces),
// the surface size and the device: operators sharing the translation kernel
// over the same trees compress with the same bases.  Oldest dropped past
// GRAM_CACHE_BYTES.
struct GramEntry {
    std::vector<double> gi, go, ev;
};
using GramKey = std::tuple<uint64_t, uint64_t, int, int>;
constexpr size_t GRAM_CACHE_BYTES = 512u << 20;
std::map<GramKey, GramEntry> gram_cache;
std::vector<GramKey> gram_cache_order;
size_t gram_cache_bytes = 0;
}  // namespace

void clear_setup_cache()
{
    std::lock_guard<std::mutex> lock(c2e_cache_mu);
    c2e_cache.clear();
    c2e_cache_order.clear();
    c2e_cache_bytes = 0;
    gram_cache.clear();
    gram_cache_order.clear();
    gram_cache_bytes = 0;
}

void Plan::build_c2e(Form& F)
{
    const Tree* trees[2] = {stree, &otree};
    double r_eq[2] = {F.r_ue, F.r_de}, r_ck[2] = {F.r_uc, F.r_dc};
    std::vector<SurfJob> jobs;       // systems factored directly
    std::vector<long> job_dst;       // their c2e offsets
    struct Scaled { long src, dst; double s; };
    std::vector<Scaled> scaled;      // levels derived from a factored one
    std::vector<long>* offs[2] = {&F.c2e_up_off, &F.c2e_dn_off};
    const long nn = (long)n * n;
    const int deg = sdim == 3 ? kernel_degree(F.g_kid) : 1;
    long total = 0;
    for (int w = 0; w < 2; w++) {
        offs[w]->clear();
        const Tree& t = *trees[w];
        const double sep = std::fabs(r_ck[w] - r_eq[w]);
        long base_off = -1;
        double base_r = 0;
        for (int l = 0; l < t.n_levels(); l++) {
            int c = t.first_at_level[l];
            const Cell& cc = t.cells[c];
            double r = hypot_ref(cc.hw);
            offs[w]->push_back(total);
            const bool scalable = deg <= 0 && r * sep > 1e-5;
            if (scalable && base_off >= 0) {
                scaled.push_back({base_off, total, std::pow(r / base_r, -(double)deg)});
            } else {
                SurfJob J;
                for (int d = 0; d < 3; d++) J.tc[d] = J.sc[d] = cc.center[d];
                J.tr = J.sr = r;
                J.trref = r_ck[w];
                J.srref = r_eq[w];
                J.out_off = (long)jobs.size() * nn;
                jobs.push_back(J);
                job_dst.push_back(total);
                if (scalable) {
                    base_off = total;
                    base_r = r;
                }
            }
            total += nn;
        }
    }
    F.c2e.alloc(total);
    if (jobs.empty()) return;
    int device = 0;
    TBEM_CK(cudaGetDevice(&device));
    const uint64_t unit_hash = hash_doubles(unit);
    auto key_of = [&](const SurfJob& J) {
        return C2EKey(F.g_kid, sdim, ns, mu, nu, J.tr, J.trref, J.srref, J.tc[0], J.tc[1], J.tc[2],
                      opt.svd_threshold, unit_hash, device);
    };
    {
        // levels factored before: copied in, the rest factored below
        std::lock_guard<std::mutex> lock(c2e_cache_mu);
        std::vector<SurfJob> todo;
        std::vector<long> todo_dst;
        for (size_t k = 0; k < jobs.size(); k++) {
            auto it = c2e_cache.find(key_of(jobs[k]));
            if (it != c2e_cache.end() && (long)it->second.size() == nn) {
                TBEM_CK(cudaMemcpyAsync(F.c2e.p + job_dst[k], it->second.data(), sizeof(double) * nn,
                                        cudaMemcpyHostToDevice, stream));
            } else {
                SurfJob J = jobs[k];
                J.out_off = (long)todo.size() * nn;
                todo.push_back(J);
                todo_dst.push_back(job_dst[k]);
            }
        }
        TBEM_CK(cudaStreamSynchronize(stream));
        jobs.swap(todo);
        job_dst.swap(todo_dst);
    }
    if (jobs.empty()) {
        for (const Scaled& sc : scaled) {
            scale_copy_kernel<<<(unsigned)std::min<long>((nn + 255) / 256, 4096), 256, 0, stream>>>(
                F.c2e.p + sc.src, F.c2e.p + sc.dst, nn, sc.s);
            TBEM_CK(cudaGetLastError());
        }
        TBEM_CK(cudaStreamSynchronize(stream));
        return;
    }
    DBuf<double> sys;
    sys.alloc(jobs.size() * nn);
    DBuf<SurfJob> dj;
    dj.alloc(jobs.size());
    TBEM_CK(cudaMemcpy(dj.p, jobs.data(), jobs.size() * sizeof(SurfJob), cudaMemcpyHostToDevice));
    TBEM_CK(cudaStreamSynchronize(cudaStreamLegacy));
    dim3 g((unsigned)((ns * ns + 255) / 256), (unsigned)jobs.size());
    surf_matrix_kernel<<<g, 256, 0, stream>>>(dj.p, d_unit.p, ns, F.g_kid,
                                               make_kparams(F.g_kid, mu, nu), sys.p);
    TBEM_CK(cudaGetLastError());
    int lwork = 0;
    TBEM_CKS(cusolverDnDgesvd_bufferSize(solver, n, n, &lwork));
    DBuf<double> work, S, U, VT;
    DBuf<int> info;
    work.alloc(std::max(lwork, 1));
    S.alloc(n);
    U.alloc(nn);
    VT.alloc(nn);
    info.alloc(1);
    for (size_t k = 0; k < jobs.size(); k++) {
        double* A = sys.p + jobs[k].out_off;
        // the row-major system seen column-major is A^T = U S V^T; the
        // row-major result pinv(A) is V^T^T-times-scaled-U^T in column-major
        char ju = 'A', jv = 'A';
        TBEM_CKS(cusolverDnDgesvd(solver, ju, jv, n, n, A, n, S.p, U.p, n, VT.p, n, work.p, lwork,
                                  nullptr, info.p));
        pinv_scale_kernel<<<n, 256, 0, stream>>>(U.p, S.p, n, opt.svd_threshold);
        TBEM_CK(cudaGetLastError());
        const double one = 1.0, zero = 0.0;
        TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_T, CUBLAS_OP_T, n, n, n, &one, VT.p, n, U.p, n, &zero,
                             F.c2e.p + job_dst[k], n));
        int h_info = 0;
        TBEM_CK(cudaMemcpyAsync(&h_info, info.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
        TBEM_CK(cudaStreamSynchronize(stream));
        if (h_info != 0)
            throw Error(TBEM_ERR_CUDA, "cuSOLVER gesvd did not converge (info " +
                                           std::to_string(h_info) + ")");
        std::vector<double> h(nn);
        TBEM_CK(cudaMemcpy(h.data(), F.c2e.p + job_dst[k], sizeof(double) * nn, cudaMemcpyDeviceToHost));
        std::lock_guard<std::mutex> lock(c2e_cache_mu);
        const C2EKey key = key_of(jobs[k]);
        if (c2e_cache.count(key)) continue;
        while (!c2e_cache_order.empty() && c2e_cache_bytes + sizeof(double) * nn > C2E_CACHE_BYTES) {
            c2e_cache_bytes -= sizeof(double) * c2e_cache[c2e_cache_order.front()].size();
            c2e_cache.erase(c2e_cache_order.front());
            c2e_cache_order.erase(c2e_cache_order.begin());
        }
        c2e_cache[key] = std::move(h);
        c2e_cache_order.push_back(key);
        c2e_cache_bytes += sizeof(double) * nn;
    }
    for (const Scaled& sc : scaled) {
        scale_copy_kernel<<<(unsigned)std::min<long>((nn + 255) / 256, 4096), 256, 0, stream>>>(
            F.c2e.p + sc.src, F.c2e.p + sc.dst, nn, sc.s);
        TBEM_CK(cudaGetLastError());
    }
    TBEM_CK(cudaStreamSynchronize(stream));
}

void Plan::build_form()
{
    Form& F = f;
    // the FP64 compressed form is the precision form's construction in FP64
    F.mixed = opt.precision == TBEM_PRECISION_MIXED || opt.precision == TBEM_PRECISION_FP64_COMPRESSED;
    F.f64 = opt.precision == TBEM_PRECISION_FP64_COMPRESSED;
    if (!F.mixed) {
        // reference radii (cpp/fmm.h:42-66) and the operator's own kernel everywhere
        const double far = 4.0 - std::sqrt(2) - 2 * cfg.d;
        F.r_ue = 0.3;
        F.r_uc = far;
        F.r_dc = 0.3;
        F.r_de = far;
        F.g_kid = F.ks_kid = F.kt_kid = kid;
    } else {
        // enclosing surfaces: the down-check sphere contains the cell, so the
        // local field is interpolated, never extrapolated, and the combined
        // operators stay O(1).  Equivalent sources are single-layer (Laplace
        // single layer / Kelvin displacement): the far field of every kernel
        // here is a harmonic potential or a Navier displacement field, which
        // single-layer densities represent; the traction kernels as their own
        // equivalent kernel converge poorly on enclosing spheres.
        F.r_ue = 1.1;
        F.r_uc = 2.9;
        F.r_dc = 1.1;
        F.r_de = 2.9;
        const bool elastic = kid == EL_DISP || kid == EL_TRAC || kid == EL_ADJ || kid == EL_HYP;
        F.g_kid = kid == IDENT ? IDENT : (elastic ? EL_DISP : LAP_S);
        // adjoint traction: point-force sources, traction observed at the
        // targets; hypersingular: dislocation sources (the traction kernel's
        // displacement field), traction observed at the targets
        F.ks_kid = kid == EL_ADJ ? EL_DISP : kid == EL_HYP ? EL_TRAC : kid;
        F.kt_kid = (kid == EL_ADJ || kid == EL_HYP) ? EL_ADJ : F.g_kid;
    }
    build_c2e(F);
    setup_mark("c2e");
    if (F.mixed) {
        build_mixed_ops(F);  // marks "translations" and "compression" inside
        setup_mark("leaf_operators");
    } else {
        build_plain_ops(F);
        setup_mark("operators");
    }
}

namespace {

// The kernel-matrix jobs of the dedup'd translations (M2M / L2L octant
// operators and M2L offsets) at the radii of a form.
void translation_jobs(const Plan& P, const Form& F, std::vector<SurfJob>& jobs,
                      std::vector<long>& m2m_off, std::vector<long>& l2l_off,
                      std::vector<long>& m2l_off, long nn)
{
    const Tree& S = *P.stree;
    const Tree& O = P.otree;
    long total = 0;
    auto add = [&](const Cell& t, double trr, const Cell& s, double srr) {
        SurfJob J;
        for (int d = 0; d < 3; d++) { J.tc[d] = t.center[d]; J.sc[d] = s.center[d]; }
        J.tr = hypot_ref(t.hw);
        J.sr = hypot_ref(s.hw);
        J.trref = trr;
        J.srref = srr;
        J.out_off = total;
        jobs.push_back(J);
        total += nn;
        return J.out_off;
    };
    // In the precision form the combined operators (kernel matrix times the
    // pseudo-inverse) do not depend on the level: every kernel here is
    // homogeneous, the surfaces of level l + 1 are those of level l scaled by
    // exactly 1/2 (cells halve, cpp/geometry.cpp:20-28), and the thresholded
    // pseudo-inverse of lambda A is pinv(A) / lambda.  Below the root (whose
    // box is the expanded one) one representative per octant / per (level
    // difference, offset) serves every level.
    const bool merge = F.mixed;
    m2m_off.assign(P.m2m_canon.size(), -1);
    std::map<int, long> m2m_rep;
    for (size_t k = 0; k < P.m2m_canon.size(); k++) {
        if (P.m2m_canon[k].first < 0) continue;  // (parent, child): up-check(parent) <- up-equiv(child)
        const int lev = (int)k / 8, oct = (int)k % 8;
        if (merge && lev >= 1 && m2m_rep.count(oct)) { m2m_off[k] = m2m_rep[oct]; continue; }
        m2m_off[k] = add(S.cells[P.m2m_canon[k].first], F.r_uc, S.cells[P.m2m_canon[k].second], F.r_ue);
        if (merge && lev >= 1) m2m_rep[oct] = m2m_off[k];
    }
    l2l_off.assign(P.l2l_canon.size(), -1);
    std::map<int, long> l2l_rep;
    for (size_t k = 0; k < P.l2l_canon.size(); k++) {
        if (P.l2l_canon[k].first < 0) continue;  // (parent, child): down-check(child) <- down-equiv(parent)
        const int lev = (int)k / 8, oct = (int)k % 8;
        if (merge && lev >= 1 && l2l_rep.count(oct)) { l2l_off[k] = l2l_rep[oct]; continue; }
        l2l_off[k] = add(O.cells[P.l2l_canon[k].second], F.r_dc, O.cells[P.l2l_canon[k].first], F.r_de);
        if (merge && lev >= 1) l2l_rep[oct] = l2l_off[k];
    }
    m2l_off.assign(P.m2l_canon.size(), -1);
    std::map<std::tuple<int, long, long, long>, long> m2l_rep;
    for (size_t k = 0; k < P.m2l_canon.size(); k++) {  // down-check(obs) <- up-equiv(src)
        const Cell& o = O.cells[P.m2l_canon[k].first];
        const Cell& sc = S.cells[P.m2l_canon[k].second];
        std::tuple<int, long, long, long> key;
        const bool mergeable = merge && o.level >= 1 && sc.level >= 1;
        if (mergeable) {
            const double* hf = o.level >= sc.level ? o.hw : sc.hw;
            long off[3];
            for (int d = 0; d < 3; d++)
                off[d] = hf[d] == 0.0 ? 0 : (long)std::nearbyint((sc.center[d] - o.center[d]) / hf[d]);
            key = std::make_tuple(o.level - sc.level, off[0], off[1], off[2]);
            auto it = m2l_rep.find(key);
            if (it != m2l_rep.end()) { m2l_off[k] = it->second; continue; }
        }
        m2l_off[k] = add(o, F.r_dc, sc, F.r_ue);
        if (mergeable) m2l_rep[key] = m2l_off[k];
    }
}

}  // namespace

void Plan::build_gemm_sets(Form& F, long, long, long, const std::vector<long>& m2m_off,
                           const std::vector<long>& l2l_off, const std::vector<long>& m2l_off)
{
    const Tree& S = *stree;
    const Tree& O = otree;
    const int LS = S.n_levels(), LO = O.n_levels();
    auto swap_pairs = [](const std::vector<std::pair<int, int>>& v) {
        std::vector<std::pair<int, int>> o(v.size());
        for (size_t i = 0; i < v.size(); i++) o[i] = {v[i].second, v[i].first};
        return o;
    };
    F.m2m.clear();
    F.m2m.resize(std::max(LS, 0));
    F.m2m_t.clear();
    F.m2m_t.resize(std::max(LS, 0));
    for (int l = 0; l < LS; l++)
        for (int o = 0; o < 8; o++) {
            int key = l * 8 + o;
            if (m2m_off[key] < 0) continue;
            F.m2m[l].add_group(m2m_off[key], m2m_pairs[key]);
            F.m2m_t[l].add_group(m2m_off[key], swap_pairs(m2m_pairs[key]));
        }
    F.l2l.clear();
    F.l2l.resize(std::max(LO, 0));
    F.l2l_t.clear();
    F.l2l_t.resize(std::max(LO, 0));
    for (int l = 0; l < LO; l++)
        for (int o = 0; o < 8; o++) {
            int key = l * 8 + o;
            if (l2l_off[key] < 0) continue;
            F.l2l[l].add_group(l2l_off[key], l2l_pairs[key]);
            F.l2l_t[l].add_group(l2l_off[key], swap_pairs(l2l_pairs[key]));
        }
    F.m2l = GemmSet();
    F.m2l_t = GemmSet();
    // keys that share an operator form one group (an observation cell still
    // appears at most once per group: its level and offset fix the key)
    std::map<long, std::vector<std::pair<int, int>>> by_op;
    std::vector<long> op_order;
    for (size_t k = 0; k < m2l_groups.size(); k++) {
        auto& pr = by_op[m2l_off[k]];
        if (pr.empty()) op_order.push_back(m2l_off[k]);
        for (int pi : m2l_groups[k]) pr.push_back({L.m2l[pi].src, L.m2l[pi].obs});
    }
    for (long off : op_order) {
        F.m2l.add_group(off, by_op[off]);
        F.m2l_t.add_group(off, swap_pairs(by_op[off]));
    }
    const void* pool = F.mixed ? (const void*)F.ops32.p : (const void*)F.ops64.p;
    const size_t esz = F.mixed ? sizeof(float) : sizeof(double);
    for (auto& g : F.m2m) g.upload(pool, esz);
    for (auto& g : F.m2m_t) g.upload(pool, esz);
    for (auto& g : F.l2l) g.upload(pool, esz);
    for (auto& g : F.l2l_t) g.upload(pool, esz);
    F.m2l.upload(pool, esz);
    F.m2l_t.upload(pool, esz);
    if (!F.mixed) {
        // the plain form's M2L through slots, at most ~1 GB of slots per RHS
        const long cap = std::max<long>(1, (1L << 30) / (8L * n));
        F.m2l_slots.build(F.m2l, cap, pool, esz);
        F.m2l_t_slots.build(F.m2l_t, cap, pool, esz);
    }
    // check-to-equivalent products, one group per level (FP64 pool)
    F.c2e_up.clear();
    F.c2e_up.resize(LS);
    F.c2e_up_t.clear();
    F.c2e_up_t.resize(LS);
    for (int l = 0; l < LS; l++) {
        std::vector<std::pair<int, int>> pr;
        for (int c = S.level_start[l]; c < S.level_start[l + 1]; c++) pr.push_back({c, c});
        F.c2e_up[l].add_group(F.c2e_up_off[l], pr);
        F.c2e_up_t[l].add_group(F.c2e_up_off[l], pr);
        F.c2e_up[l].upload(F.c2e.p, sizeof(double));
        F.c2e_up_t[l].upload(F.c2e.p, sizeof(double));
    }
    F.c2e_dn.clear();
    F.c2e_dn.resize(LO);
    F.c2e_dn_t.clear();
    F.c2e_dn_t.resize(LO);
    for (int l = 0; l < LO; l++) {
        std::vector<std::pair<int, int>> pr;
        for (int c = O.level_start[l]; c < O.level_start[l + 1]; c++) pr.push_back({c, c});
        F.c2e_dn[l].add_group(F.c2e_dn_off[l], pr);
        F.c2e_dn_t[l].add_group(F.c2e_dn_off[l], pr);
        F.c2e_dn[l].upload(F.c2e.p, sizeof(double));
        F.c2e_dn_t[l].upload(F.c2e.p, sizeof(double));
    }
}

void Plan::build_plain_ops(Form& F)
{
    const long nn = (long)n * n;
    std::vector<SurfJob> jobs;
    std::vector<long> m2m_off, l2l_off, m2l_off;
    translation_jobs(*this, F, jobs, m2m_off, l2l_off, m2l_off, nn);
    F.ops64.alloc(std::max<long>((long)jobs.size() * nn, 1));
    if (!jobs.empty()) {
        DBuf<SurfJob> dj;
        dj.alloc(jobs.size());
        TBEM_CK(cudaMemcpy(dj.p, jobs.data(), jobs.size() * sizeof(SurfJob), cudaMemcpyHostToDevice));
        TBEM_CK(cudaStreamSynchronize(cudaStreamLegacy));
        for (size_t j0 = 0; j0 < jobs.size(); j0 += 32768) {
            unsigned nj = (unsigned)std::min<size_t>(32768, jobs.size() - j0);
            dim3 g((unsigned)((ns * ns + 255) / 256), nj);
            surf_matrix_kernel<<<g, 256, 0, stream>>>(dj.p + j0, d_unit.p, ns, F.g_kid,
                                                       make_kparams(F.g_kid, mu, nu), F.ops64.p);
            TBEM_CK(cudaGetLastError());
        }
        TBEM_CK(cudaStreamSynchronize(stream));
    }
    build_gemm_sets(F, 0, 0, 0, m2m_off, l2l_off, m2l_off);
}

void Plan::build_mixed_ops(Form& F)
{
    const long nn = (long)n * n;
    std::vector<SurfJob> jobs;
    std::vector<long> m2m_off, l2l_off, m2l_off;
    translation_jobs(*this, F, jobs, m2m_off, l2l_off, m2l_off, nn);
    const long total = (long)jobs.size() * nn;
    F.ops32.alloc(std::max<long>(total, 1));
    const double one = 1.0, zero = 0.0;
    // combined operator of job k: K_k * C2E(level of the k-th operator's source side)
    std::vector<long> c2e_of(jobs.size(), -1);
    std::vector<int> job_ls(jobs.size(), 0);  // M2L jobs: source level they were built at
    {
        const Tree& S = *stree;
        const Tree& O = otree;
        // the pseudo-inverse of the level the operator's job was built at (the
        // first key that uses a job is the one that created it)
        for (size_t k = 0; k < m2m_off.size(); k++)
            if (m2m_off[k] >= 0 && c2e_of[m2m_off[k] / nn] < 0)
                c2e_of[m2m_off[k] / nn] = F.c2e_up_off[S.cells[m2m_canon[k].second].level];
        for (size_t k = 0; k < l2l_off.size(); k++)
            if (l2l_off[k] >= 0 && c2e_of[l2l_off[k] / nn] < 0)
                c2e_of[l2l_off[k] / nn] = F.c2e_dn_off[O.cells[l2l_canon[k].first].level];
        for (size_t k = 0; k < m2l_off.size(); k++)
            if (c2e_of[m2l_off[k] / nn] < 0) {
                c2e_of[m2l_off[k] / nn] = F.c2e_up_off[S.cells[m2l_canon[k].second].level];
                job_ls[m2l_off[k] / nn] = S.cells[m2l_canon[k].second].level;
            }
    }
    // m2l_path: 0 auto (= 5 where the M2L operators are precomputed and
    // compress, else SIMT FP32),
    // 1 SIMT FP32 for all, 2 tensor cores for the M2L only, 3 tensor cores for
    // all, 4 compressed, 5 compressed with the M2L products on tensor cores
    // (the FP64 compressed form: compressed, FP64 SIMT)
    const int path = F.f64 ? 4 : opt.m2l_path == 0 ? 5 : opt.m2l_path;
    // FP64 copies of the M2L kernel matrices for the compression (compact
    // index), scaled to the root level (see build_m2l_compression)
    const bool compress = (path == 4 || path == 5) && !F.m2l_on_the_fly && !m2l_off.empty();
    std::vector<long> m2l_index(jobs.size(), -1);
    long n_m2l_ops = 0;
    for (long off : m2l_off)
        if (off >= 0 && m2l_index[off / nn] < 0) m2l_index[off / nn] = n_m2l_ops++;
    // and of the M2M kernel matrices / combined L2L operators (compact; the
    // first key of a job is the one that built it)
    std::vector<long> m2m_index(jobs.size(), -1), l2l_index(jobs.size(), -1);
    std::vector<int> m2m_lc;
    long n_m2m_ops = 0, n_l2l_ops = 0;
    for (size_t k = 0; k < m2m_off.size(); k++)
        if (m2m_off[k] >= 0 && m2m_index[m2m_off[k] / nn] < 0) {
            m2m_index[m2m_off[k] / nn] = n_m2m_ops++;
            m2m_lc.push_back(stree->cells[m2m_canon[k].second].level);
        }
    for (size_t k = 0; k < l2l_off.size(); k++)
        if (l2l_off[k] >= 0 && l2l_index[l2l_off[k] / nn] < 0) l2l_index[l2l_off[k] / nn] = n_l2l_ops++;
    DBuf<double> U64, KM, YL;
    if (compress) {
        U64.alloc((size_t)n_m2l_ops * nn);
        KM.alloc(std::max<long>(n_m2m_ops, 1) * nn);
        YL.alloc(std::max<long>(n_l2l_ops, 1) * nn);
    }
    // The kernel matrices of every job, and the combined operators K C2E:
    // `dense` fills the FP32 pool with all of them (the uncompressed paths);
    // without it only the L2L jobs' combined operators are formed, the
    // compression taking the M2L and M2M jobs' kernel matrices alone (each
    // skipped product is 2 n^3 FP64 flops).  `copies` saves the compression's
    // inputs.
    auto build_jobs = [&](bool dense, bool copies) {
        if (jobs.empty()) return;
        // in chunks to bound the FP64 scratch
        // (one grid row per job: at most 65,535 jobs per chunk)
        const size_t chunk = std::min<size_t>(65535, std::max<size_t>(1, (size_t)(2e9 / (8.0 * nn))));
        DBuf<SurfJob> dj;
        DBuf<double> K, Y;
        K.alloc(std::min(chunk, jobs.size()) * nn);
        Y.alloc(std::min(chunk, jobs.size()) * nn);
        for (size_t j0 = 0; j0 < jobs.size(); j0 += chunk) {
            size_t nj = std::min(chunk, jobs.size() - j0);
            std::vector<SurfJob> sub(jobs.begin() + j0, jobs.begin() + j0 + nj);
            for (size_t k = 0; k < nj; k++) sub[k].out_off = (long)k * nn;
            dj.alloc(nj);
            TBEM_CK(cudaMemcpy(dj.p, sub.data(), nj * sizeof(SurfJob), cudaMemcpyHostToDevice));
            TBEM_CK(cudaStreamSynchronize(cudaStreamLegacy));
            dim3 g((unsigned)((ns * ns + 255) / 256), (unsigned)nj);
            surf_matrix_kernel<<<g, 256, 0, stream>>>(dj.p, d_unit.p, ns, F.g_kid,
                                                       make_kparams(F.g_kid, mu, nu), K.p);
            TBEM_CK(cudaGetLastError());
            for (size_t k = 0; k < nj; k++) {
                if (!dense && l2l_index[j0 + k] < 0) continue;
                // row-major Y = K * C  <=>  column-major Y^T = C^T K^T
                TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one,
                                     F.c2e.p + c2e_of[j0 + k], n, K.p + k * nn, n, &zero,
                                     Y.p + k * nn, n));
            }
            if (dense) {
                convert_kernel<float><<<grid_for(nj * nn), 256, 0, stream>>>(Y.p, F.ops32.p + j0 * nn, nj * nn);
                TBEM_CK(cudaGetLastError());
            }
            if (copies)
                for (size_t k = 0; k < nj; k++) {
                    if (m2l_index[j0 + k] >= 0) {
                        double* dst = U64.p + m2l_index[j0 + k] * nn;
                        TBEM_CK(cudaMemcpyAsync(dst, K.p + k * nn, sizeof(double) * nn,
                                                cudaMemcpyDeviceToDevice, stream));
                        const double f = std::ldexp(1.0, -job_ls[j0 + k]);
                        TBEM_CKB(cublasDscal(cublas, (int)nn, &f, dst, 1));
                    }
                    if (m2m_index[j0 + k] >= 0)
                        TBEM_CK(cudaMemcpyAsync(KM.p + m2m_index[j0 + k] * nn, K.p + k * nn, sizeof(double) * nn,
                                                cudaMemcpyDeviceToDevice, stream));
                    if (l2l_index[j0 + k] >= 0)
                        TBEM_CK(cudaMemcpyAsync(YL.p + l2l_index[j0 + k] * nn, Y.p + k * nn, sizeof(double) * nn,
                                                cudaMemcpyDeviceToDevice, stream));
                }
            TBEM_CK(cudaStreamSynchronize(stream));
        }
    };
    build_jobs(!compress, compress);
    build_gemm_sets(F, 0, 0, 0, m2m_off, l2l_off, m2l_off);
    setup_mark("translations");
    F.m2l_compressed = false;
    if (compress) {
        CompressionInput in{U64.p, n_m2l_ops, &m2l_index, KM.p, &m2m_lc, &m2m_index,
                            YL.p, &l2l_index, &m2m_off, &l2l_off, {0, 0}};
        // what the root-scaled M2L matrices depend on, in compact order
        const uint64_t bases[2] = {1469598103934665603ull, 0x9e3779b97f4a7c15ull};
        const uint64_t uh = hash_doubles(unit);
        const double prm[2] = {mu, nu};
        const int ints[3] = {F.g_kid, ns, sdim};
        for (int h = 0; h < 2; h++) {
            uint64_t k = hash_bytes(ints, sizeof(ints), bases[h]);
            k = hash_bytes(prm, sizeof(prm), k);
            k = hash_bytes(&uh, sizeof(uh), k);
            k = hash_bytes(&n_m2l_ops, sizeof(n_m2l_ops), k);
            std::vector<long> order(n_m2l_ops, -1);
            for (size_t j = 0; j < jobs.size(); j++)
                if (m2l_index[j] >= 0) order[m2l_index[j]] = (long)j;
            for (long j : order) {
                const SurfJob& J = jobs[j];
                const double g[10] = {J.tc[0], J.tc[1], J.tc[2], J.tr, J.trref,
                                      J.sc[0], J.sc[1], J.sc[2], J.sr, J.srref};
                k = hash_bytes(g, sizeof(g), k);
                k = hash_bytes(&job_ls[j], sizeof(int), k);
            }
            in.t0_key[h] = k;
        }
        build_compression(F, in);
    }
    U64.release();
    KM.release();
    YL.release();
    // the compression declined: the dense combined operators after all
    if (compress && !F.m2l_compressed && !F.f64) build_jobs(true, false);
    if (F.f64 && !F.m2l_compressed)
        throw Error(TBEM_ERR_ARG, "the FP64 compressed form needs M2L operators that compress (the "
                                  "compressed products cheaper than the dense ones)");
    if (F.m2l_compressed && path == 5) {
        F.use_tc_c = true;
        F.tc_c.build(F.Cops.p, n_m2l_ops, F.r_out, F.r_in, stream);
        TBEM_CK(cudaStreamSynchronize(stream));
    }
    // the auto path keeps the M2L products on the tensor cores when they do
    // not compress (uncompressed 3xBF16 planes)
    const bool auto_tc = opt.m2l_path == 0 && !F.f64 && !F.m2l_compressed && !F.m2l_on_the_fly &&
                         !m2l_off.empty();
    F.use_tc = (path == 2 || path == 3 || auto_tc) && !jobs.empty();
    F.use_tc_updown = F.use_tc && path == 3;
    if (F.use_tc) {
        F.tc.build(F.ops32.p, (long)jobs.size(), n, n, stream);
        TBEM_CK(cudaStreamSynchronize(stream));
    }
    setup_mark("compression");

    // per-leaf L2P operators E = K(points, down-equiv) * C2E_down(level)
    const Tree& O = otree;
    std::vector<int> leaves(L.l2p.begin(), L.l2p.end());
    std::stable_sort(leaves.begin(), leaves.end(),
                     [&](int a, int b) { return O.cells[a].level < O.cells[b].level; });
    std::vector<long> row0, pt0;
    std::vector<int> cell, npts;
    long rows = 0;
    for (int c : leaves) {
        const Cell& cc = O.cells[c];
        if (cc.n_points() == 0) continue;
        row0.push_back(rows);
        pt0.push_back(cc.pt_begin);
        cell.push_back(c);
        npts.push_back((int)cc.n_points());
        rows += cc.n_points() * R;
    }
    F.n_l2p = (int)cell.size();
    // compressed form: E V, taking the r_out downward coefficients directly
    const int ecols = F.m2l_compressed ? F.r_out : n;
    F.E_ld = (ecols + 127) / 128 * 128;
    if (F.E_ld > 2048) throw Error(TBEM_ERR_ARG, "translation surface too large for the L2P kernel");
    if (F.f64) F.E64.alloc(std::max<long>(rows * F.E_ld, 1));
    else F.E.alloc(std::max<long>(rows * F.E_ld, 1));
    auto store_rows = [&](const double* src, long off, long r, int cols) {
        if (F.f64)
            convert_rows_kernel<double><<<grid_for(r * F.E_ld), 256, 0, stream>>>(src, F.E64.p + off, r, cols, F.E_ld);
        else
            convert_rows_kernel<float><<<grid_for(r * F.E_ld), 256, 0, stream>>>(src, F.E.p + off, r, cols, F.E_ld);
    };
    F.E_row0.upload(row0);
    F.E_pt0.upload(pt0);
    F.E_leaf.upload(cell);
    F.E_npts.upload(npts);
    if (rows > 0) {
        const long max_rows = std::max<long>((long)R * 64, (long)(1.5e9 / (8.0 * n)));
        DBuf<double> K, Y, EV, CV;
        // compressed form: E V = K (C2E_down(level) V), the n x r_out factor
        // formed once per level -- 2 r r_out n flops per chunk of r rows
        // where (K C2E) V took 2 r n (n + r_out), and the setup's FP64 GEMMs
        // run at about 1.25 TFLOP/s on this part
        if (F.m2l_compressed) CV.alloc((size_t)n * F.r_out);
        int cv_level = -1;
        // chunks of consecutive leaves of one level
        size_t t0 = 0;
        while (t0 < cell.size()) {
            const int lev = O.cells[cell[t0]].level;
            size_t t1 = t0;
            long r = 0;
            // (one grid row per leaf: at most 65,535 leaves per chunk)
            while (t1 < cell.size() && O.cells[cell[t1]].level == lev && t1 - t0 < 65535 &&
                   (r + (long)npts[t1] * R <= max_rows || t1 == t0)) {
                r += (long)npts[t1] * R;
                t1++;
            }
            K.ensure(r * n);
            int maxp = 0;
            for (size_t t = t0; t < t1; t++) maxp = std::max(maxp, npts[t]);
            dim3 g((unsigned)(((long)maxp * ns + 255) / 256), (unsigned)(t1 - t0));
            pts_surf_matrix_kernel<<<g, 256, 0, stream>>>(
                F.E_pt0.p + t0, F.E_npts.p + t0, F.E_leaf.p + t0, F.E_row0.p + t0, dobs.xyz.p,
                dobs.nrm64.p, dobs.center.p, dobs.rad.p, F.r_de, d_unit.p, ns, F.kt_kid,
                make_kparams(F.kt_kid, mu, nu), K.p, row0[t0]);
            TBEM_CK(cudaGetLastError());
            if (F.m2l_compressed) {
                // column-major CV = C^T V (C the stored pseudo-inverse, its
                // column-major transpose being the row-major operator), then
                // row-major E V (r x r_out) = column-major CV^T K^T
                if (lev != cv_level) {
                    TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_T, CUBLAS_OP_N, n, F.r_out, n, &one,
                                         F.c2e.p + F.c2e_dn_off[lev], n, F.V64.p, n, &zero, CV.p, n));
                    cv_level = lev;
                }
                EV.ensure(r * F.r_out);
                TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_T, CUBLAS_OP_N, F.r_out, (int)r, n, &one, CV.p, n,
                                     K.p, n, &zero, EV.p, F.r_out));
                store_rows(EV.p, row0[t0] * F.E_ld, r, F.r_out);
            } else {
                Y.ensure(r * n);
                TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, (int)r, n, &one,
                                     F.c2e.p + F.c2e_dn_off[lev], n, K.p, n, &zero, Y.p, n));
                store_rows(Y.p, row0[t0] * F.E_ld, r, n);
            }
            TBEM_CK(cudaGetLastError());
            TBEM_CK(cudaStreamSynchronize(stream));
            t0 = t1;
        }
    }
    F.V64.release();
}

// The compressed precision form.  The bases are those of SVD-compressed M2L
// (Fong & Darve, J. Comput. Phys. 228 (2009) 8712-8725, sec. 3.3), taken from
// the M2L kernel matrices T (down-check surface of the target <- up-
// equivalent surface of the source), not from the combined operators
// T C2E_up: the pseudo-inverse magnifies directions the check potentials
// never carry, which would make those look full rank.  Both translation
// kernels are homogeneous of degree -1, so a pair at source level l_s has
// T = 2^l_s T0 with T0 the root-scaled matrix of its (level difference,
// offset) class, and
//   T C2E_up(l_s) = T0 (2^l_s C2E_up(l_s)) ~= V (V^T T0 W) (W^T 2^l_s C2E_up(l_s))
//                 = V C_k P_(l_s),
// W the leading eigenvectors of sum_k T0_k^T T0_k (input side), V those of
// sum_k T0_k T0_k^T (output side), cut where the eigenvalue falls below
// tol^2 times the largest (singular values of the stacks below tol times the
// largest).  r_out is rounded up to the GEMM's 64-row tile and r_in to its
// 16-deep k step: the extra vectors cost nothing in the products.
//
// The whole far field then lives in these bases.  A source cell carries
// u~ = P_l u (u its up-check potentials): its root-scaled equivalent density
// q0 = 2^l C2E_up(l) u seen through W.  The M2M of child c (level l_c) into
// parent p (level l_p) adds K q_c to the parent's check potentials (K the
// kernel matrix parent up-check <- child up-equivalent), with
// q_c ~= 2^-l_c W u~_c, so u~_p += X u~_c with X = P_(l_p) K W 2^-l_c.
// Dropping the part of q_c outside W is what the M2L drops as well: a
// translation to a farther, larger cell only maps expansion content of a
// given order into content of the same or higher order.  A target cell
// carries d~ with its down-check potentials d ~= V d~; the L2L combined
// operator L (child down-check <- parent down-check) becomes V^T L V and the
// L2P operator E of a leaf becomes E V.  Source points reaching a target's
// down-check surface directly (P2L) enter through V^T; the equivalent
// densities of an M2P source are 2^-l W u~.
void Plan::build_compression(Form& F, const CompressionInput& in)
{
    if (F.g_kid != LAP_S && F.g_kid != EL_DISP)
        throw Error(TBEM_ERR_STATE, "compressed form needs a degree -1 translation kernel");
    const long nn = (long)n * n;
    const double one = 1.0, zero = 0.0;
    const double tol = opt.m2l_rank_tol > 0 ? opt.m2l_rank_tol : 1e-7;
    const double* T0 = in.T0;
    const long n_ops = in.n_m2l;
    DBuf<double> Gi, Go;
    Gi.alloc(nn);
    Go.alloc(nn);
    DBuf<double> ev;
    ev.alloc(2 * (size_t)n);
    int device = 0;
    TBEM_CK(cudaGetDevice(&device));
    const GramKey gkey(in.t0_key[0], in.t0_key[1], n, device);
    std::vector<double> h_ev;
    {
        std::lock_guard<std::mutex> lock(c2e_cache_mu);
        auto it = gram_cache.find(gkey);
        if (it != gram_cache.end()) {
            TBEM_CK(cudaMemcpyAsync(Gi.p, it->second.gi.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, stream));
            TBEM_CK(cudaMemcpyAsync(Go.p, it->second.go.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, stream));
            TBEM_CK(cudaStreamSynchronize(stream));
            h_ev = it->second.ev;
        }
    }
    if (h_ev.empty()) {
        // G (+)= A A^T for A = kb n x n blocks side by side (column-major
        // n x kb n).  A small n leaves the product a few output tiles for the
        // whole k = kb n, most SMs idle: there the blocks are cut into groups
        // whose products run as one strided-batched GEMM, summed by a GEMV.
        constexpr long GRAM_GROUPS = 64;
        DBuf<double> part, ones;
        if (n <= 512) {
            part.alloc((size_t)GRAM_GROUPS * nn);
            std::vector<double> h1(GRAM_GROUPS, 1.0);
            ones.upload(h1);
        }
        auto gram_add = [&](const double* A, long kb, double* G, bool first) {
            const double beta = first ? 0.0 : 1.0;
            if (n > 512 || kb < 2 * GRAM_GROUPS) {
                TBEM_CKB(cublasDsyrk(cublas, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, n, (int)(kb * n), &one, A, n,
                                     &beta, G, n));
                return;
            }
            const long gk = kb / GRAM_GROUPS, rem = kb - GRAM_GROUPS * gk;
            TBEM_CKB(cublasDgemmStridedBatched(cublas, CUBLAS_OP_N, CUBLAS_OP_T, n, n, (int)(gk * n), &one, A, n,
                                               (long long)(gk * nn), A, n, (long long)(gk * nn), &zero, part.p, n,
                                               (long long)nn, (int)GRAM_GROUPS));
            TBEM_CKB(cublasDgemv(cublas, CUBLAS_OP_N, (int)nn, (int)GRAM_GROUPS, &one, part.p, (int)nn, ones.p, 1,
                                 &beta, G, 1));
            if (rem > 0)
                TBEM_CKB(cublasDsyrk(cublas, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, n, (int)(rem * n), &one,
                                     A + GRAM_GROUPS * gk * nn, n, &one, G, n));
        };
        // G_in = sum_k T_k^T T_k = X X^T, X = [T_1^T ... T_K^T]: the column-major
        // view of the row-major matrices side by side (chunks bound the int sizes)
        const long step = std::max<long>(1, (1L << 30) / std::max(nn, 1L));
        for (long k0 = 0; k0 < n_ops; k0 += step)
            gram_add(T0 + k0 * nn, std::min(step, n_ops - k0), Gi.p, k0 == 0);
        // G_out = sum_k T_k T_k^T: chunks of the matrices transposed side by
        // side (column-major n x kb n = [T_1 ... T_kb], 256 MB of staging) and
        // one rank-(kb n) update per chunk instead of one rank-n update per
        // matrix
        const long tstep = std::max<long>(1, std::min<long>(step, (256L << 20) / (long)sizeof(double) / nn));
        DBuf<double> Tt;
        Tt.alloc((size_t)std::min(tstep, n_ops) * nn);
        for (long k0 = 0; k0 < n_ops; k0 += tstep) {
            const long kb = std::min(tstep, n_ops - k0);
            transpose_blocks_kernel<<<grid_for(kb * nn), 256, 0, stream>>>(T0 + k0 * nn, Tt.p, n, kb);
            TBEM_CK(cudaGetLastError());
            gram_add(Tt.p, kb, Go.p, k0 == 0);
        }
        // eigenvectors (ascending eigenvalues) overwrite the Gram matrices
        int lwork = 0;
        TBEM_CKS(cusolverDnDsyevd_bufferSize(solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n,
                                             Gi.p, n, ev.p, &lwork));
        DBuf<double> work;
        work.alloc(std::max(lwork, 1));
        DBuf<int> info;
        info.alloc(2);
        TBEM_CKS(cusolverDnDsyevd(solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, Gi.p, n,
                                  ev.p, work.p, lwork, info.p));
        TBEM_CKS(cusolverDnDsyevd(solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, Go.p, n,
                                  ev.p + n, work.p, lwork, info.p + 1));
        h_ev = ev.download();
        std::vector<int> h_info = info.download();
        if (h_info[0] != 0 || h_info[1] != 0)
            throw Error(TBEM_ERR_CUDA, "eigen-decomposition of the M2L Gram matrices failed");
        GramEntry e{Gi.download(), Go.download(), h_ev};
        std::lock_guard<std::mutex> lock(c2e_cache_mu);
        if (!gram_cache.count(gkey)) {
            const size_t bytes = sizeof(double) * (e.gi.size() + e.go.size() + e.ev.size());
            while (!gram_cache_order.empty() && gram_cache_bytes + bytes > GRAM_CACHE_BYTES) {
                const GramEntry& old = gram_cache[gram_cache_order.front()];
                gram_cache_bytes -= sizeof(double) * (old.gi.size() + old.go.size() + old.ev.size());
                gram_cache.erase(gram_cache_order.front());
                gram_cache_order.erase(gram_cache_order.begin());
            }
            gram_cache[gkey] = std::move(e);
            gram_cache_order.push_back(gkey);
            gram_cache_bytes += bytes;
        }
    }
    auto rank_of = [&](const double* e) {
        const double top = e[n - 1];
        int r = 0;
        for (int i = 0; i < n; i++)
            if (e[i] > tol * tol * top) r++;
        return std::max(r, 1);
    };
    const int ri = std::min(n, (rank_of(h_ev.data()) + 15) / 16 * 16);
    const int ro = std::min(n, (rank_of(h_ev.data() + n) + 63) / 64 * 64);
    // no gain once the compressed products, padded to the tensor-core tiles
    // (128 output rows, 64-deep K chunks), cost as much as the dense ones
    auto pad = [](long v, long q) { return (v + q - 1) / q * q; };
    if (pad(ro, 128) * pad(ri, 64) >= pad(n, 128) * pad(n, 64) || (long)ri * ro > nn * 9 / 10) return;
    F.r_in = ri;
    F.r_out = ro;
    const double* W = Gi.p + (long)(n - ri) * n;  // column-major n x ri
    const double* V = Go.p + (long)(n - ro) * n;  // column-major n x ro
    F.V64.alloc((size_t)n * ro);
    TBEM_CK(cudaMemcpyAsync(F.V64.p, V, sizeof(double) * n * ro, cudaMemcpyDeviceToDevice, stream));
    // the operator pools: FP32 (the precision form) or FP64 (the FP64
    // compressed form); `store` copies count FP64 values into one of them
    const bool f64 = F.f64;
    auto store = [&](const double* src, long count, DBuf<float>& p32, DBuf<double>& p64, long off) {
        if (count <= 0) return;
        if (f64) convert_kernel<double><<<grid_for(count), 256, 0, stream>>>(src, p64.p + off, count);
        else convert_kernel<float><<<grid_for(count), 256, 0, stream>>>(src, p32.p + off, count);
        TBEM_CK(cudaGetLastError());
    };
    auto alloc_pool = [&](size_t count, DBuf<float>& p32, DBuf<double>& p64) {
        if (f64) p64.alloc(count);
        else p32.alloc(count);
    };
    alloc_pool((size_t)n * ro, F.Vb, F.Vb64);
    if (f64) basis_rows_kernel<double><<<grid_for((long)n * ro), 256, 0, stream>>>(Go.p, n, ro, 1.0, F.Vb64.p);
    else basis_rows_kernel<float><<<grid_for((long)n * ro), 256, 0, stream>>>(Go.p, n, ro, 1.0, F.Vb.p);
    TBEM_CK(cudaGetLastError());
    const Tree& S = *stree;
    const Tree& O = otree;
    const int LS = S.n_levels(), LO = O.n_levels();
    // P_l = 2^l W^T C2E_up(l), row-major ri x n = the column-major n x ri
    // product 2^l C2E_up(l)^T W (C2E_up(l)^T being the column-major view of
    // the stored operator); kept in FP64 for the M2M operators
    DBuf<double> P64;
    P64.alloc((size_t)LS * n * ri);
    alloc_pool((size_t)LS * n * ri, F.Pb, F.Pb64);
    alloc_pool((size_t)LS * n * ri, F.Wl, F.Wl64);
    for (int l = 0; l < LS; l++) {
        const double f = std::ldexp(1.0, l);
        TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, ri, n, &f, F.c2e.p + F.c2e_up_off[l], n, W,
                             n, &zero, P64.p + (long)l * n * ri, n));
        if (f64)
            basis_rows_kernel<double><<<grid_for((long)n * ri), 256, 0, stream>>>(
                Gi.p, n, ri, std::ldexp(1.0, -l), F.Wl64.p + (long)l * n * ri);
        else
            basis_rows_kernel<float><<<grid_for((long)n * ri), 256, 0, stream>>>(
                Gi.p, n, ri, std::ldexp(1.0, -l), F.Wl.p + (long)l * n * ri);
        TBEM_CK(cudaGetLastError());
    }
    store(P64.p, (long)LS * n * ri, F.Pb, F.Pb64, 0);
    // C_k (row-major ro x ri) = column-major C_k^T = W^T T_k^T V, T_k^T being
    // the column-major view of the stored matrix
    const long cc = (long)ro * ri;
    alloc_pool((size_t)n_ops * cc, F.Cops, F.Cops64);
    const long cb = std::max<long>(1, std::min<long>(n_ops, (long)(1e9 / (8.0 * n * ro))));
    const long n_m2m = (long)in.m2m_lc->size();
    long n_l2l = 0;
    for (long v : *in.l2l_index) n_l2l = std::max(n_l2l, v + 1);
    DBuf<double> P, CT;
    P.alloc((size_t)cb * n * std::max(ro, ri));
    CT.alloc((size_t)std::max(cb * cc, std::max(n_m2m * ri * ri, n_l2l * ro * ro)));
    for (long k0 = 0; k0 < n_ops; k0 += cb) {
        const long kb = std::min(cb, n_ops - k0);
        TBEM_CKB(cublasDgemmStridedBatched(cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, ro, n, &one,
                                           T0 + k0 * nn, n, nn, V, n, 0, &zero, P.p, n,
                                           (long long)n * ro, (int)kb));
        TBEM_CKB(cublasDgemmStridedBatched(cublas, CUBLAS_OP_T, CUBLAS_OP_N, ri, ro, n, &one, W, n, 0,
                                           P.p, n, (long long)n * ro, &zero, CT.p, ri, cc, (int)kb));
        store(CT.p, kb * cc, F.Cops, F.Cops64, k0 * cc);
        TBEM_CK(cudaStreamSynchronize(stream));
    }
    // X (row-major ri x ri) = column-major X^T = 2^-l_c W^T (K^T P_(l_p)^T)
    alloc_pool(std::max<long>(n_m2m, 1) * ri * ri, F.Xops, F.Xops64);
    for (long j = 0; j < n_m2m; j++) {
        const int lc = (*in.m2m_lc)[j], lp = lc - 1;
        const double f = std::ldexp(1.0, -lc);
        TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, ri, n, &one, in.KM + j * nn, n,
                             P64.p + (long)lp * n * ri, n, &zero, P.p, n));
        TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_T, CUBLAS_OP_N, ri, ri, n, &f, W, n, P.p, n, &zero,
                             CT.p + j * (long)ri * ri, ri));
    }
    store(CT.p, n_m2m * ri * ri, F.Xops, F.Xops64, 0);
    TBEM_CK(cudaStreamSynchronize(stream));
    // Y (row-major ro x ro) = column-major Y^T = V^T (L^T V), L^T the
    // column-major view of the combined operator
    alloc_pool(std::max<long>(n_l2l, 1) * ro * ro, F.Yops, F.Yops64);
    for (long j = 0; j < n_l2l; j++) {
        TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_N, CUBLAS_OP_N, n, ro, n, &one, in.YL + j * nn, n, V, n,
                             &zero, P.p, n));
        TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_T, CUBLAS_OP_N, ro, ro, n, &one, V, n, P.p, n, &zero,
                             CT.p + j * (long)ro * ro, ro));
    }
    store(CT.p, n_l2l * ro * ro, F.Yops, F.Yops64, 0);
    TBEM_CK(cudaStreamSynchronize(stream));

    // GEMM sets.  M2L: F.m2l's groups on the C_k pool.
    auto swap_pairs = [](const std::vector<std::pair<int, int>>& v) {
        std::vector<std::pair<int, int>> o(v.size());
        for (size_t i = 0; i < v.size(); i++) o[i] = {v[i].second, v[i].first};
        return o;
    };
    F.m2l_c = GemmSet();
    F.m2l_c_t = GemmSet();
    for (size_t g = 0; g < F.m2l.A_off.size(); g++) {
        std::vector<std::pair<int, int>> pr;
        for (long p = F.m2l.pair0[g]; p < F.m2l.pair0[g] + F.m2l.npairs[g]; p++)
            pr.push_back({F.m2l.in_cell[p], F.m2l.out_cell[p]});
        const long idx = (*in.m2l_index)[F.m2l.A_off[g] / nn];
        if (idx < 0) throw Error(TBEM_ERR_STATE, "M2L operator without a compressed copy");
        F.m2l_c.add_group(idx * cc, pr);
        F.m2l_c_t.add_group(idx * cc, swap_pairs(pr));
    }
    // M2M / L2L per level and octant on the X / Y pools, pruned to the pairs
    // that reach a result: an upward state is used only if the cell or an
    // ancestor is an M2L / M2P source, a downward state is nonzero only if the
    // cell or an ancestor receives M2L / P2L (levels are parent-first)
    std::vector<char> up_used(S.cells.size(), 0), down_used(O.cells.size(), 0);
    for (size_t p = 0; p < F.m2l.in_cell.size(); p++) {
        up_used[F.m2l.in_cell[p]] = 1;
        down_used[F.m2l.out_cell[p]] = 1;
    }
    for (const auto& pr : L.m2p) up_used[pr.src] = 1;
    for (const auto& pr : L.p2l) down_used[pr.obs] = 1;
    for (size_t c = 0; c < S.cells.size(); c++)
        if (S.cells[c].parent >= 0 && up_used[S.cells[c].parent]) up_used[c] = 1;
    for (size_t c = 0; c < O.cells.size(); c++)
        if (O.cells[c].parent >= 0 && down_used[O.cells[c].parent]) down_used[c] = 1;
    auto keep_out = [](const std::vector<std::pair<int, int>>& v, const std::vector<char>& used) {
        std::vector<std::pair<int, int>> o;
        for (const auto& q : v)
            if (used[q.second]) o.push_back(q);  // (child, parent): the parent's state is used
        return o;
    };
    auto keep_in = [](const std::vector<std::pair<int, int>>& v, const std::vector<char>& used) {
        std::vector<std::pair<int, int>> o;
        for (const auto& q : v)
            if (used[q.first]) o.push_back(q);   // (parent, child): the parent's state is nonzero
        return o;
    };
    F.m2m_c.clear();
    F.m2m_c.resize(std::max(LS, 0));
    F.m2m_c_t.clear();
    F.m2m_c_t.resize(std::max(LS, 0));
    for (int l = 0; l < LS; l++)
        for (int o = 0; o < 8; o++) {
            const int key = l * 8 + o;
            const long off = (*in.m2m_off)[key];
            if (off < 0) continue;
            const long idx = (*in.m2m_index)[off / nn];
            const auto pr = keep_out(m2m_pairs[key], up_used);
            F.m2m_c[l].add_group(idx * ri * ri, pr);
            F.m2m_c_t[l].add_group(idx * ri * ri, swap_pairs(pr));
        }
    F.l2l_c.clear();
    F.l2l_c.resize(std::max(LO, 0));
    F.l2l_c_t.clear();
    F.l2l_c_t.resize(std::max(LO, 0));
    for (int l = 0; l < LO; l++)
        for (int o = 0; o < 8; o++) {
            const int key = l * 8 + o;
            const long off = (*in.l2l_off)[key];
            if (off < 0) continue;
            const long idx = (*in.l2l_index)[off / nn];
            const auto pr = keep_in(l2l_pairs[key], down_used);
            F.l2l_c[l].add_group(idx * ro * ro, pr);
            F.l2l_c_t[l].add_group(idx * ro * ro, swap_pairs(pr));
        }
    // compress the P2M cells (P_l per level), rebuild the densities of the M2P
    // sources (2^-l W per level), move the P2L targets through V
    F.comp_p2m = GemmSet();
    F.decomp_m2p = GemmSet();
    F.comp_p2l = GemmSet();
    std::vector<char> is_p2m(S.cells.size(), 0), is_m2p(S.cells.size(), 0), is_p2l(O.cells.size(), 0);
    for (int c : L.p2m) is_p2m[c] = 1;
    for (const auto& pr : L.m2p) is_m2p[pr.src] = 1;
    for (const auto& pr : L.p2l) is_p2l[pr.obs] = 1;
    for (int l = 0; l < LS; l++) {
        std::vector<std::pair<int, int>> a, b;
        for (int c = S.level_start[l]; c < S.level_start[l + 1]; c++) {
            if (is_p2m[c] && up_used[c]) a.push_back({c, c});
            if (is_m2p[c]) b.push_back({c, c});
        }
        F.comp_p2m.add_group((long)l * n * ri, a);
        F.decomp_m2p.add_group((long)l * n * ri, b);
    }
    {
        std::vector<std::pair<int, int>> a;
        for (int c = 0; c < (int)O.cells.size(); c++)
            if (is_p2l[c]) a.push_back({c, c});
        F.comp_p2l.add_group(0, a);
    }
    F.decomp_l2p = GemmSet();
    {
        std::vector<std::pair<int, int>> a;
        for (int c : L.l2p) a.push_back({c, c});
        F.decomp_l2p.add_group(0, a);
    }
    // the sets resolve their operators in the pool of the form's precision
    const size_t es = f64 ? sizeof(double) : sizeof(float);
    auto pool = [&](DBuf<float>& p32, DBuf<double>& p64) -> const void* {
        return f64 ? static_cast<const void*>(p64.p) : static_cast<const void*>(p32.p);
    };
    F.m2l_c.upload(pool(F.Cops, F.Cops64), es);
    F.m2l_c_t.upload(pool(F.Cops, F.Cops64), es);
    for (auto& g : F.m2m_c) g.upload(pool(F.Xops, F.Xops64), es);
    for (auto& g : F.m2m_c_t) g.upload(pool(F.Xops, F.Xops64), es);
    for (auto& g : F.l2l_c) g.upload(pool(F.Yops, F.Yops64), es);
    for (auto& g : F.l2l_c_t) g.upload(pool(F.Yops, F.Yops64), es);
    F.comp_p2m.upload(pool(F.Pb, F.Pb64), es);
    F.decomp_m2p.upload(pool(F.Wl, F.Wl64), es);
    F.comp_p2l.upload(pool(F.Vb, F.Vb64), es);
    F.decomp_l2p.upload(pool(F.Vb, F.Vb64), es);
    F.m2l_compressed = true;
}

void Plan::set_c2e(int which, long level, const double* op)
{
    if (opt.host_only) throw Error(TBEM_ERR_STATE, "operator was built with host_only");
    DeviceGuard guard(opt.device);
    if (f.mixed) throw Error(TBEM_ERR_STATE, "set_c2e is only valid for the FP64 form");
    const auto& offs = which == 0 ? f.c2e_up_off : f.c2e_dn_off;
    if (level < 0 || level >= (long)offs.size()) throw Error(TBEM_ERR_ARG, "level out of range");
    TBEM_CK(cudaStreamSynchronize(stream));
    TBEM_CK(cudaMemcpy(f.c2e.p + offs[level], op, (size_t)n * n * sizeof(double),
                       cudaMemcpyHostToDevice));
    TBEM_CK(cudaStreamSynchronize(cudaStreamLegacy));
}

void Plan::get_c2e(int which, long level, double* out) const
{
    if (opt.host_only) throw Error(TBEM_ERR_STATE, "operator was built with host_only");
    DeviceGuard guard(opt.device);
    const auto& offs = which == 0 ? f.c2e_up_off : f.c2e_dn_off;
    if (level < 0 || level >= (long)offs.size()) throw Error(TBEM_ERR_ARG, "level out of range");
    TBEM_CK(cudaStreamSynchronize(stream));
    TBEM_CK(cudaMemcpy(out, f.c2e.p + offs[level], (size_t)n * n * sizeof(double),
                       cudaMemcpyDeviceToHost));
}

// ------------------------------------------------------------------ apply

void Plan::ensure_rhs(int nrhs)
{
    if (nrhs <= cap_rhs) return;
    const long ncs = (long)stree->cells.size(), nco = (long)otree.cells.size();
    const long N = std::max(n_obs, n_src);
    io_x.ensure((size_t)R * std::max<long>(n_src, n_obs) * nrhs);
    io_y.ensure((size_t)R * N * nrhs);
    s64.ensure((size_t)R * N * nrhs);
    y64.ensure((size_t)R * N * nrhs);
    if (f.f64) {
        // the FP64 compressed form: check potentials, coefficients, M2P densities
        cu64.ensure((size_t)ncs * nrhs * n);
        if (!L.p2l.empty()) cd64.ensure((size_t)nco * nrhs * n);
        cuc64.ensure((size_t)ncs * nrhs * f.r_in);
        cdc64.ensure((size_t)nco * nrhs * f.r_out);
        if (!L.m2p.empty()) qu64.ensure((size_t)ncs * nrhs * n);
    } else if (f.mixed) {
        s32.ensure((size_t)R * N * nrhs);
        cu32.ensure((size_t)ncs * nrhs * n);
        cd32.ensure((size_t)nco * nrhs * n);
        if (f.m2l_compressed) {
            cuc32.ensure((size_t)ncs * nrhs * f.r_in);
            cdc32.ensure((size_t)nco * nrhs * f.r_out);
        }
        if (!L.m2p.empty() || f.m2l_on_the_fly) {
            cu64.ensure((size_t)ncs * nrhs * n);
            qu64.ensure((size_t)ncs * nrhs * n);
            cd64.ensure((size_t)nco * nrhs * n);
        }
    } else {
        cu64.ensure((size_t)ncs * nrhs * n);
        qu64.ensure((size_t)ncs * nrhs * n);
        cd64.ensure((size_t)nco * nrhs * n);
        qd64.ensure((size_t)nco * nrhs * n);
        const long slots = std::max(f.m2l_slots.max_slots, f.m2l_t_slots.max_slots);
        if (slots > 0) slots64.ensure((size_t)slots * nrhs * n);
    }
    cap_rhs = nrhs;
}

// The precision form's L2P of `nrhs` right-hand sides from the per-leaf
// states cd ([cell][rhs][len]): one right-hand side at a time streams the
// leaf operators E once per right-hand side; from two on, E is read once per
// block of L2P_NRB.
template <typename T>
void Plan::launch_l2p(const T* cd, int len, int nrhs, cudaStream_t s)
{
    Form& F = f;
    const size_t smem = sizeof(T) * (size_t)F.E_ld * L2P_NRB;
    const T* E;
    if constexpr (sizeof(T) == 4) E = F.E.p; else E = F.E64.p;
    if ((nrhs > 1 || sizeof(T) == 8) && smem <= 200 * 1024) {
        if (smem > 48 * 1024 && smem > l2p_smem_set[sizeof(T) / 8]) {
            TBEM_CK(cudaFuncSetAttribute(l2p_multi_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
            l2p_smem_set[sizeof(T) / 8] = smem;
        }
        l2p_multi_kernel<T><<<F.n_l2p, L2P_MULTI_THREADS, smem, s>>>(
            E, F.E_row0.p, F.E_leaf.p, F.E_pt0.p, F.E_npts.p, cd, len, F.E_ld, R, nrhs, y64.p, n_obs);
    } else if constexpr (sizeof(T) == 4) {
        l2p_mixed_kernel<<<F.n_l2p, 256, 0, s>>>(E, F.E_row0.p, F.E_leaf.p, F.E_pt0.p, F.E_npts.p, cd,
                                                  len, F.E_ld, R, nrhs, y64.p, n_obs);
    } else {
        throw Error(TBEM_ERR_ARG, "translation surface too large for the FP64 L2P kernel");
    }
    TBEM_CK(cudaGetLastError());
    launches++;
}

void Plan::mark(const char* name, cudaStream_t s)
{
    if (!timing) return;
    cudaEvent_t e;
    if (!event_pool.empty()) {
        e = event_pool.back();
        event_pool.pop_back();
    } else {
        TBEM_CK(cudaEventCreate(&e));
    }
    TBEM_CK(cudaEventRecord(e, s));
    marks.push_back({name, e});
}

namespace {
double steady_seconds()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

void Plan::setup_start()
{
    setup_s.clear();
    setup_t = steady_seconds();
}

void Plan::setup_mark(const char* name)
{
    if (!opt.host_only && stream) TBEM_CK(cudaStreamSynchronize(stream));
    const double t = steady_seconds();
    setup_s.push_back({name, t - setup_t});
    setup_t = t;
}

void Plan::read_phases()
{
    if (marks.empty()) return;
    DeviceGuard guard(opt.device);
    TBEM_CK(cudaEventSynchronize(marks.back().second));
    std::vector<std::pair<std::string, double>> sum;
    int applies = 0;
    for (size_t i = 0; i < marks.size(); i++) {
        // "apply" opens an apply; "start" a right-hand-side chunk of it (the
        // copies and the time between chunks belong to no phase)
        if (marks[i].first == "apply") {
            applies++;
            continue;
        }
        if (marks[i].first == "start") continue;
        if (i == 0) continue;
        float ms = 0.f;
        TBEM_CK(cudaEventElapsedTime(&ms, marks[i - 1].second, marks[i].second));
        auto it = std::find_if(sum.begin(), sum.end(), [&](const auto& q) { return q.first == marks[i].first; });
        if (it == sum.end()) sum.push_back({marks[i].first, ms});
        else it->second += ms;
    }
    for (auto& q : sum) q.second /= std::max(applies, 1);
    phase_ms = sum;
    for (auto& m : marks) event_pool.push_back(m.second);
    marks.clear();
}

template <typename T>
void Plan::eval(const TaskSet& ts, int ekid, bool tgt_surf, bool src_surf, const Tree&,
                const DTree& dt, double t_rref, const DTree& ds, double s_rref, const T* s_str,
                long s_n, const T* q, double* y, long y_n, T* c, int add, int nrhs,
                cudaStream_t s, bool trans)
{
    if (ts.n_items() == 0) return;
    EvalArgs<T> a{};
    ts.fill(a);
    a.t_xyz = dt.xyz.p;
    if constexpr (sizeof(T) == 4) a.t_nrm = dt.nrm32.p; else a.t_nrm = dt.nrm64.p;
    a.t_center = dt.center.p;
    a.t_rad = dt.rad.p;
    a.t_rref = t_rref;
    a.s_xyz = ds.xyz.p;
    if constexpr (sizeof(T) == 4) a.s_nrm = ds.nrm32.p; else a.s_nrm = ds.nrm64.p;
    a.s_nrm64 = ds.nrm64.p;
    a.s_str = s_str;
    a.s_n = s_n;
    a.s_center = ds.center.p;
    a.s_rad = ds.rad.p;
    a.s_rref = s_rref;
    a.q = q;
    a.unit = d_unit.p;
    a.ns = ns;
    a.y = y;
    a.y_n = y_n;
    a.c = c;
    a.nrhs = nrhs;
    a.add = add;
    const KParams ep = make_kparams(ekid, mu, nu);
    a.c2 = T(ep.c2);
    a.scale = ep.scale;
    EvalLaunch Lc{ekid, trans, tgt_surf, src_surf, ts.n_items()};
    Lc.tpt = ts.tpt;
    for (int r0 = 0; r0 < nrhs; r0 += eval_rhs_block(ekid, sizeof(T) == 4, trans, src_surf, nrhs - r0)) {
        a.rhs0 = r0;
        TBEM_CK(launch_eval<T>(Lc, a, s));
        launches++;
    }
}

void Plan::forward(int nrhs, cudaStream_t s)
{
    const Tree& S = *stree;
    const Tree& O = otree;
    const long NS = n_src, NO = n_obs;
    const long ncs = (long)S.cells.size(), nco = (long)O.cells.size();
    Form& F = f;
    mark("start", s);
    TBEM_CK(cudaMemsetAsync(y64.p, 0, sizeof(double) * R * NO * nrhs, s));
    if (F.mixed && F.m2l_compressed) {
        if (F.f64) forward_compressed<double>(nrhs, s);
        else forward_compressed<float>(nrhs, s);
    } else if (!F.mixed) {
        gather_kernel<double><<<grid_for(NS * R * nrhs), 256, 0, s>>>(xin, dsrc->perm.p, dsrc->w.p, s64.p, NS, R, nrhs);
        TBEM_CK(cudaGetLastError());
        launches++;
        TBEM_CK(cudaMemsetAsync(cu64.p, 0, sizeof(double) * ncs * nrhs * n, s));
        TBEM_CK(cudaMemsetAsync(cd64.p, 0, sizeof(double) * nco * nrhs * n, s));
        mark("gather", s);
        eval<double>(p2m_set(), F.ks_kid, true, false, S, *dsrc, F.r_uc, *dsrc, 0, s64.p, NS, nullptr, nullptr, 0, cu64.p, 0, nrhs, s, false);
        mark("p2m", s);
        for (int l = S.n_levels() - 1; l >= 0; l--) {
            if (l < (int)F.m2m.size()) F.m2m[l].run<double>(qu64.p, cu64.p, n, nrhs, 0, GEMM_WAVES, s, &launches);
            F.c2e_up[l].run<double>(cu64.p, qu64.p, n, nrhs, 0, GEMM_STORE, s, &launches);
        }
        mark("m2m+c2e_up", s);
        eval<double>(p2p_set(), kid, false, false, O, dobs, 0, *dsrc, 0, s64.p, NS, nullptr, y64.p, NO, nullptr, 1, nrhs, s, false);
        mark("p2p", s);
        eval<double>(m2p, F.kt_kid, false, true, O, dobs, 0, *dsrc, F.r_ue, nullptr, 0, qu64.p, y64.p, NO, nullptr, 1, nrhs, s, false);
        eval<double>(p2l, F.ks_kid, true, false, O, dobs, F.r_dc, *dsrc, 0, s64.p, NS, nullptr, nullptr, 0, cd64.p, 1, nrhs, s, false);
        mark("m2p+p2l", s);
        if (F.m2l_on_the_fly)
            eval<double>(m2l_fly, F.g_kid, true, true, O, dobs, F.r_dc, *dsrc, F.r_ue, nullptr, 0, qu64.p, nullptr, 0, cd64.p, 1, nrhs, s, false);
        else
            F.m2l_slots.run(qu64.p, cd64.p, n, nrhs, 0, slots64.p, s, &launches);
        mark("m2l", s);
        for (int l = 0; l < O.n_levels(); l++) {
            if (l > 0 && l - 1 < (int)F.l2l.size()) F.l2l[l - 1].run<double>(qd64.p, cd64.p, n, nrhs, 0, GEMM_ADD, s, &launches);
            F.c2e_dn[l].run<double>(cd64.p, qd64.p, n, nrhs, 0, GEMM_STORE, s, &launches);
        }
        mark("l2l+c2e_down", s);
        eval<double>(l2p, F.kt_kid, false, true, O, dobs, 0, dobs, F.r_de, nullptr, 0, qd64.p, y64.p, NO, nullptr, 1, nrhs, s, false);
        mark("l2p", s);
    } else {
        gather_kernel<float><<<grid_for(NS * R * nrhs), 256, 0, s>>>(xin, dsrc->perm.p, dsrc->w.p, s32.p, NS, R, nrhs);
        TBEM_CK(cudaGetLastError());
        launches++;
        TBEM_CK(cudaMemsetAsync(cu32.p, 0, sizeof(float) * ncs * nrhs * n, s));
        TBEM_CK(cudaMemsetAsync(cd32.p, 0, sizeof(float) * nco * nrhs * n, s));
        mark("gather", s);
        eval<float>(p2m_set(), F.ks_kid, true, false, S, *dsrc, F.r_uc, *dsrc, 0, s32.p, NS, nullptr, nullptr, 0, cu32.p, 0, nrhs, s, false);
        mark("p2m", s);
        for (int l = S.n_levels() - 1; l >= 0; l--) {
            if (l >= (int)F.m2m.size() || F.m2m[l].empty()) continue;
            if (F.use_tc_updown) {
                // children of level l live at level l + 1 (contiguous cells)
                const long r0 = (long)S.level_start[l + 1] * nrhs;
                const long rn = (long)(S.level_start[l + 2] - S.level_start[l + 1]) * nrhs;
                F.tc.split_b_rows(cu32.p, r0, rn, ncs * nrhs, s);
                launches++;
                F.m2m[l].run_tc(F.tc, cu32.p, nrhs, 1, (long)n * n, s, &launches);
            } else {
                F.m2m[l].run<float>(cu32.p, cu32.p, n, nrhs, 0, GEMM_ATOMIC, s, &launches);
            }
        }
        mark("m2m", s);
        eval<float>(p2p_set(), kid, false, false, O, dobs, 0, *dsrc, 0, s32.p, NS, nullptr, y64.p, NO, nullptr, 1, nrhs, s, false);
        mark("p2p", s);
        const bool need64 = !L.m2p.empty() || F.m2l_on_the_fly;
        if (need64) {
            // explicit equivalent densities in FP64 (see the form notes)
            promote_kernel<<<grid_for(ncs * nrhs * n), 256, 0, s>>>(cu32.p, cu64.p, ncs * nrhs * n);
            TBEM_CK(cudaGetLastError());
            launches++;
            for (int l = 0; l < S.n_levels(); l++) F.c2e_up[l].run<double>(cu64.p, qu64.p, n, nrhs, 0, GEMM_STORE, s, &launches);
            eval<double>(m2p, F.kt_kid, false, true, O, dobs, 0, *dsrc, F.r_ue, nullptr, 0, qu64.p, y64.p, NO, nullptr, 1, nrhs, s, false);
        }
        eval<float>(p2l, F.ks_kid, true, false, O, dobs, F.r_dc, *dsrc, 0, s32.p, NS, nullptr, nullptr, 0, cd32.p, 1, nrhs, s, false);
        mark("m2p+p2l", s);
        if (F.m2l_on_the_fly) {
            TBEM_CK(cudaMemsetAsync(cd64.p, 0, sizeof(double) * nco * nrhs * n, s));
            eval<double>(m2l_fly, F.g_kid, true, true, O, dobs, F.r_dc, *dsrc, F.r_ue, nullptr, 0, qu64.p, nullptr, 0, cd64.p, 1, nrhs, s, false);
            add_kernel<<<grid_for(nco * nrhs * n), 256, 0, s>>>(cd64.p, cd32.p, nco * nrhs * n);
            TBEM_CK(cudaGetLastError());
            launches++;
        } else if (F.use_tc) {
            F.tc.split_b_rows(cu32.p, 0, ncs * nrhs, std::max(ncs, nco) * nrhs, s);
            launches++;
            F.m2l.run_tc(F.tc, cd32.p, nrhs, 1, (long)n * n, s, &launches);
        } else {
            F.m2l.run<float>(cu32.p, cd32.p, n, nrhs, 0, GEMM_ATOMIC, s, &launches);
        }
        mark("m2l", s);
        for (int l = 1; l < O.n_levels(); l++) {
            if (l - 1 >= (int)F.l2l.size() || F.l2l[l - 1].empty()) continue;
            if (F.use_tc_updown) {
                // parents at level l - 1 (contiguous cells)
                const long r0 = (long)O.level_start[l - 1] * nrhs;
                const long rn = (long)(O.level_start[l] - O.level_start[l - 1]) * nrhs;
                F.tc.split_b_rows(cd32.p, r0, rn, std::max(ncs, nco) * nrhs, s);
                launches++;
                F.l2l[l - 1].run_tc(F.tc, cd32.p, nrhs, 0, (long)n * n, s, &launches);
            } else {
                F.l2l[l - 1].run<float>(cd32.p, cd32.p, n, nrhs, 0, GEMM_ADD, s, &launches);
            }
        }
        mark("l2l", s);
        if (F.n_l2p > 0) launch_l2p(cd32.p, n, nrhs, s);
        mark("l2p", s);
    }
    scatter_kernel<<<grid_for(NO * R * nrhs), 256, 0, s>>>(y64.p, dobs.perm.p, nullptr, yout, NO, R, nrhs);
    TBEM_CK(cudaGetLastError());
    launches++;
    mark("scatter", s);
}

void Plan::adjoint(int nrhs, cudaStream_t s)
{
    const Tree& S = *stree;
    const Tree& O = otree;
    const long NS = n_src, NO = n_obs;
    const long ncs = (long)S.cells.size(), nco = (long)O.cells.size();
    Form& F = f;
    mark("start", s);
    // y64 holds the transposed inputs (observation space, tree order), s64 the
    // accumulated outputs (source space) before the weights
    TBEM_CK(cudaMemsetAsync(s64.p, 0, sizeof(double) * R * NS * nrhs, s));
    if (F.mixed && F.m2l_compressed) {
        if (F.f64) adjoint_compressed<double>(nrhs, s);
        else adjoint_compressed<float>(nrhs, s);
    } else if (!F.mixed) {
        gather_kernel<double><<<grid_for(NO * R * nrhs), 256, 0, s>>>(xin, dobs.perm.p, nullptr, y64.p, NO, R, nrhs);
        TBEM_CK(cudaGetLastError());
        launches++;
        TBEM_CK(cudaMemsetAsync(qu64.p, 0, sizeof(double) * ncs * nrhs * n, s));
        TBEM_CK(cudaMemsetAsync(qd64.p, 0, sizeof(double) * nco * nrhs * n, s));
        // L2P^T, M2P^T, P2P^T
        eval<double>(l2p_t, F.kt_kid, true, false, O, dobs, F.r_de, dobs, 0, y64.p, NO, nullptr, nullptr, 0, qd64.p, 1, nrhs, s, true);
        eval<double>(m2p_t, F.kt_kid, true, false, S, *dsrc, F.r_ue, dobs, 0, y64.p, NO, nullptr, nullptr, 0, qu64.p, 1, nrhs, s, true);
        eval<double>(p2p_t, kid, false, false, S, *dsrc, 0, dobs, 0, y64.p, NO, nullptr, s64.p, NS, nullptr, 1, nrhs, s, true);
        // down pass reversed: deepest level first
        for (int l = O.n_levels() - 1; l >= 0; l--) {
            F.c2e_dn_t[l].run<double>(qd64.p, cd64.p, n, nrhs, 1, GEMM_STORE, s, &launches);
            if (l > 0 && l - 1 < (int)F.l2l_t.size()) F.l2l_t[l - 1].run<double>(cd64.p, qd64.p, n, nrhs, 1, GEMM_WAVES, s, &launches);
        }
        if (F.m2l_on_the_fly)
            eval<double>(m2l_fly_t, F.g_kid, true, true, S, *dsrc, F.r_ue, dobs, F.r_dc, nullptr, 0, cd64.p, nullptr, 0, qu64.p, 1, nrhs, s, true);
        else
            F.m2l_t_slots.run(cd64.p, qu64.p, n, nrhs, 1, slots64.p, s, &launches);
        eval<double>(p2l_t, F.ks_kid, false, true, S, *dsrc, 0, dobs, F.r_dc, nullptr, 0, cd64.p, s64.p, NS, nullptr, 1, nrhs, s, true);
        // up pass reversed: root first
        for (int l = 0; l < S.n_levels(); l++) {
            F.c2e_up_t[l].run<double>(qu64.p, cu64.p, n, nrhs, 1, GEMM_STORE, s, &launches);
            if (l < (int)F.m2m_t.size()) F.m2m_t[l].run<double>(cu64.p, qu64.p, n, nrhs, 1, GEMM_ADD, s, &launches);
        }
        eval<double>(p2m_t, F.ks_kid, false, true, S, *dsrc, 0, *dsrc, F.r_uc, nullptr, 0, cu64.p, s64.p, NS, nullptr, 1, nrhs, s, true);
    } else {
        gather_kernel<float><<<grid_for(NO * R * nrhs), 256, 0, s>>>(xin, dobs.perm.p, nullptr, s32.p, NO, R, nrhs);
        TBEM_CK(cudaGetLastError());
        launches++;
        TBEM_CK(cudaMemsetAsync(cu32.p, 0, sizeof(float) * ncs * nrhs * n, s));
        TBEM_CK(cudaMemsetAsync(cd32.p, 0, sizeof(float) * nco * nrhs * n, s));
        if (F.n_l2p > 0) {
            l2p_mixed_t_kernel<float><<<F.n_l2p, 256, 0, s>>>(F.E.p, F.E_row0.p, F.E_leaf.p, F.E_pt0.p, F.E_npts.p, s32.p, NO, n, F.E_ld, R, nrhs, cd32.p);
            TBEM_CK(cudaGetLastError());
            launches++;
        }
        eval<float>(p2p_t, kid, false, false, S, *dsrc, 0, dobs, 0, s32.p, NO, nullptr, s64.p, NS, nullptr, 1, nrhs, s, true);
        const bool need64 = !L.m2p.empty() || F.m2l_on_the_fly;
        if (need64) {
            TBEM_CK(cudaMemsetAsync(qu64.p, 0, sizeof(double) * ncs * nrhs * n, s));
            // obs-space inputs in FP64 for the FP64 sub-paths
            gather_kernel<double><<<grid_for(NO * R * nrhs), 256, 0, s>>>(xin, dobs.perm.p, nullptr, y64.p, NO, R, nrhs);
            TBEM_CK(cudaGetLastError());
            launches++;
            eval<double>(m2p_t, F.kt_kid, true, false, S, *dsrc, F.r_ue, dobs, 0, y64.p, NO, nullptr, nullptr, 0, qu64.p, 1, nrhs, s, true);
        }
        for (int l = O.n_levels() - 1; l >= 1; l--)
            if (l - 1 < (int)F.l2l_t.size()) F.l2l_t[l - 1].run<float>(cd32.p, cd32.p, n, nrhs, 1, GEMM_ATOMIC, s, &launches);
        if (F.m2l_on_the_fly) {
            promote_kernel<<<grid_for(nco * nrhs * n), 256, 0, s>>>(cd32.p, cd64.p, nco * nrhs * n);
            TBEM_CK(cudaGetLastError());
            launches++;
            eval<double>(m2l_fly_t, F.g_kid, true, true, S, *dsrc, F.r_ue, dobs, F.r_dc, nullptr, 0, cd64.p, nullptr, 0, qu64.p, 1, nrhs, s, true);
        } else {
            F.m2l_t.run<float>(cd32.p, cu32.p, n, nrhs, 1, GEMM_ATOMIC, s, &launches);
        }
        if (need64) {
            // g_cup += C2E_up^T g_qup  (FP64), folded into the FP32 buffer
            for (int l = 0; l < S.n_levels(); l++) F.c2e_up_t[l].run<double>(qu64.p, cu64.p, n, nrhs, 1, GEMM_STORE, s, &launches);
            add_kernel<<<grid_for(ncs * nrhs * n), 256, 0, s>>>(cu64.p, cu32.p, ncs * nrhs * n);
            TBEM_CK(cudaGetLastError());
            launches++;
        }
        eval<float>(p2l_t, F.ks_kid, false, true, S, *dsrc, 0, dobs, F.r_dc, nullptr, 0, cd32.p, s64.p, NS, nullptr, 1, nrhs, s, true);
        for (int l = 0; l < S.n_levels(); l++)
            if (l < (int)F.m2m_t.size()) F.m2m_t[l].run<float>(cu32.p, cu32.p, n, nrhs, 1, GEMM_ADD, s, &launches);
        eval<float>(p2m_t, F.ks_kid, false, true, S, *dsrc, 0, *dsrc, F.r_uc, nullptr, 0, cu32.p, s64.p, NS, nullptr, 1, nrhs, s, true);
    }
    scatter_kernel<<<grid_for(NS * R * nrhs), 256, 0, s>>>(s64.p, dsrc->perm.p, dsrc->w.p, yout, NS, R, nrhs);
    TBEM_CK(cudaGetLastError());
    launches++;
    mark("scatter", s);
}

namespace {
// the FP32 or the FP64 buffer of a pair
template <typename T>
T* pick(DBuf<float>& a, DBuf<double>& b)
{
    if constexpr (sizeof(T) == 4) return a.p;
    else return b.p;
}
}  // namespace

// The compressed forms (see build_compression): the same passes as the
// uncompressed precision form with every cell state in the SVD bases; T =
// float for the precision form, double for the FP64 compressed form.
template <typename T>
void Plan::forward_compressed(int nrhs, cudaStream_t s)
{
    const Tree& S = *stree;
    const Tree& O = otree;
    const long NS = n_src, NO = n_obs;
    const long ncs = (long)S.cells.size(), nco = (long)O.cells.size();
    Form& F = f;
    const int ri = F.r_in, ro = F.r_out;
    T* str = pick<T>(s32, s64);
    T* cu = pick<T>(cu32, cu64);
    T* cd = pick<T>(cd32, cd64);
    T* cuc = pick<T>(cuc32, cuc64);
    T* cdc = pick<T>(cdc32, cdc64);
    gather_kernel<T><<<grid_for(NS * R * nrhs), 256, 0, s>>>(xin, dsrc->perm.p, dsrc->w.p, str, NS, R, nrhs);
    TBEM_CK(cudaGetLastError());
    launches++;
    TBEM_CK(cudaMemsetAsync(cuc, 0, sizeof(T) * ncs * nrhs * ri, s));
    TBEM_CK(cudaMemsetAsync(cdc, 0, sizeof(T) * nco * nrhs * ro, s));
    mark("gather", s);
    // the near field on the side stream, beside the far-field passes below
    TBEM_CK(cudaEventRecord(ev_fork, s));
    TBEM_CK(cudaStreamWaitEvent(side, ev_fork, 0));
    eval<T>(p2p_set(), kid, false, false, O, dobs, 0, *dsrc, 0, str, NS, nullptr, y64.p, NO, nullptr, 1, nrhs, side, false);
    TBEM_CK(cudaEventRecord(ev_join, side));
    // P2M into the leaves' check potentials, then u~ = P_l u
    eval<T>(p2m_set(), F.ks_kid, true, false, S, *dsrc, F.r_uc, *dsrc, 0, str, NS, nullptr, nullptr, 0, cu, 0, nrhs, s, false);
    F.comp_p2m.run_rect<T>(cu, cuc, ri, n, n, nrhs, 0, GEMM_ATOMIC, s, &launches);  // into zeros
    mark("p2m", s);
    for (int l = S.n_levels() - 1; l >= 0; l--)
        if (l < (int)F.m2m_c.size()) F.m2m_c[l].run_rect<T>(cuc, cuc, ri, ri, ri, nrhs, 0, GEMM_ATOMIC, s, &launches);
    mark("m2m", s);
    if (!L.p2l.empty()) {
        TBEM_CK(cudaMemsetAsync(cd, 0, sizeof(T) * nco * nrhs * n, s));
        eval<T>(p2l, F.ks_kid, true, false, O, dobs, F.r_dc, *dsrc, 0, str, NS, nullptr, nullptr, 0, cd, 1, nrhs, s, false);
        F.comp_p2l.run_rect<T>(cd, cdc, ro, n, ro, nrhs, 1, GEMM_ATOMIC, s, &launches);
    }
    mark("m2p+p2l", s);
    bool tc_done = false;
    if constexpr (sizeof(T) == 4) {
        if (F.use_tc_c) {
            F.tc_c.split_b_rows(cuc, 0, ncs * nrhs, std::max(ncs, nco) * nrhs, s);
            launches++;
            mark("m2l_split", s);
            F.m2l_c.run_tc(F.tc_c, cdc, nrhs, 1, (long)ro * ri, s, &launches);
            tc_done = true;
        }
    }
    if (!tc_done) F.m2l_c.run_rect<T>(cuc, cdc, ro, ri, ri, nrhs, 0, GEMM_ATOMIC, s, &launches);
    mark("m2l", s);
    for (int l = 1; l < O.n_levels(); l++)
        if (l - 1 < (int)F.l2l_c.size()) F.l2l_c[l - 1].run_rect<T>(cdc, cdc, ro, ro, ro, nrhs, 0, GEMM_ATOMIC, s, &launches);
    mark("l2l", s);
    // join the near field: the passes below add into the same outputs
    TBEM_CK(cudaStreamWaitEvent(s, ev_join, 0));
    mark("p2p_wait", s);
    if (!L.m2p.empty()) {
        // equivalent densities 2^-l W u~ of the M2P sources, evaluated in FP64
        F.decomp_m2p.run_rect<T>(cuc, cu, n, ri, ri, nrhs, 0, GEMM_STORE, s, &launches);
        const double* q64 = nullptr;
        if constexpr (sizeof(T) == 4) {
            promote_kernel<<<grid_for(ncs * nrhs * n), 256, 0, s>>>(cu, qu64.p, ncs * nrhs * n);
            TBEM_CK(cudaGetLastError());
            launches++;
            q64 = qu64.p;
        } else {
            q64 = cu;
        }
        eval<double>(m2p, F.kt_kid, false, true, O, dobs, 0, *dsrc, F.r_ue, nullptr, 0, q64, y64.p, NO, nullptr, 1, nrhs, s, false);
    }
    if (F.n_l2p > 0) launch_l2p<T>(cdc, ro, nrhs, s);
    mark("l2p", s);
}

template <typename T>
void Plan::adjoint_compressed(int nrhs, cudaStream_t s)
{
    const Tree& S = *stree;
    const Tree& O = otree;
    const long NS = n_src, NO = n_obs;
    const long ncs = (long)S.cells.size(), nco = (long)O.cells.size();
    Form& F = f;
    const int ri = F.r_in, ro = F.r_out;
    // the observation-side input: FP32 strengths, or (FP64 form) the FP64 buffer
    T* zin;
    if constexpr (sizeof(T) == 4) zin = s32.p; else zin = y64.p;
    T* cu = pick<T>(cu32, cu64);
    T* cd = pick<T>(cd32, cd64);
    T* cuc = pick<T>(cuc32, cuc64);
    T* cdc = pick<T>(cdc32, cdc64);
    const T* E;
    if constexpr (sizeof(T) == 4) E = F.E.p; else E = F.E64.p;
    gather_kernel<T><<<grid_for(NO * R * nrhs), 256, 0, s>>>(xin, dobs.perm.p, nullptr, zin, NO, R, nrhs);
    TBEM_CK(cudaGetLastError());
    launches++;
    TBEM_CK(cudaMemsetAsync(cuc, 0, sizeof(T) * ncs * nrhs * ri, s));
    TBEM_CK(cudaMemsetAsync(cdc, 0, sizeof(T) * nco * nrhs * ro, s));
    if (F.n_l2p > 0) {
        l2p_mixed_t_kernel<T><<<F.n_l2p, 256, 0, s>>>(E, F.E_row0.p, F.E_leaf.p, F.E_pt0.p, F.E_npts.p, zin, NO, ro, F.E_ld, R, nrhs, cdc);
        TBEM_CK(cudaGetLastError());
        launches++;
    }
    eval<T>(p2p_t, kid, false, false, S, *dsrc, 0, dobs, 0, zin, NO, nullptr, s64.p, NS, nullptr, 1, nrhs, s, true);
    for (int l = O.n_levels() - 1; l >= 1; l--)
        if (l - 1 < (int)F.l2l_c_t.size()) F.l2l_c_t[l - 1].run_rect<T>(cdc, cdc, ro, ro, ro, nrhs, 1, GEMM_ATOMIC, s, &launches);
    F.m2l_c_t.run_rect<T>(cdc, cuc, ri, ro, ri, nrhs, 1, GEMM_ATOMIC, s, &launches);
    if (!L.p2l.empty()) {
        F.comp_p2l.run_rect<T>(cdc, cd, n, ro, ro, nrhs, 0, GEMM_STORE, s, &launches);
        eval<T>(p2l_t, F.ks_kid, false, true, S, *dsrc, 0, dobs, F.r_dc, nullptr, 0, cd, s64.p, NS, nullptr, 1, nrhs, s, true);
    }
    if (!L.m2p.empty()) {
        // density gradients in FP64, folded into u~ through (2^-l W)^T
        TBEM_CK(cudaMemsetAsync(qu64.p, 0, sizeof(double) * ncs * nrhs * n, s));
        if constexpr (sizeof(T) == 4) {
            gather_kernel<double><<<grid_for(NO * R * nrhs), 256, 0, s>>>(xin, dobs.perm.p, nullptr, y64.p, NO, R, nrhs);
            TBEM_CK(cudaGetLastError());
            launches++;
        }
        eval<double>(m2p_t, F.kt_kid, true, false, S, *dsrc, F.r_ue, dobs, 0, y64.p, NO, nullptr, nullptr, 0, qu64.p, 1, nrhs, s, true);
        if constexpr (sizeof(T) == 4) {
            TBEM_CK(cudaMemsetAsync(cu, 0, sizeof(float) * ncs * nrhs * n, s));
            add_kernel<<<grid_for(ncs * nrhs * n), 256, 0, s>>>(qu64.p, cu, ncs * nrhs * n);
            TBEM_CK(cudaGetLastError());
            launches++;
            F.decomp_m2p.run_rect<float>(cu, cuc, ri, n, ri, nrhs, 1, GEMM_ATOMIC, s, &launches);
        } else {
            F.decomp_m2p.run_rect<double>(qu64.p, cuc, ri, n, ri, nrhs, 1, GEMM_ATOMIC, s, &launches);
        }
    }
    for (int l = 0; l < S.n_levels(); l++)
        if (l < (int)F.m2m_c_t.size()) F.m2m_c_t[l].run_rect<T>(cuc, cuc, ri, ri, ri, nrhs, 1, GEMM_ATOMIC, s, &launches);
    // the compression set skips the P2M leaves whose states reach no result
    // (their transposed states are zero), but the transposed P2M below reads
    // every P2M leaf: clear the buffer first (it still holds the M2P densities
    // or an earlier apply's values)
    TBEM_CK(cudaMemsetAsync(cu, 0, sizeof(T) * ncs * nrhs * n, s));
    F.comp_p2m.run_rect<T>(cuc, cu, n, ri, n, nrhs, 1, GEMM_STORE, s, &launches);
    eval<T>(p2m_t, F.ks_kid, false, true, S, *dsrc, 0, *dsrc, F.r_uc, nullptr, 0, cu, s64.p, NS, nullptr, 1, nrhs, s, true);
}

void Plan::apply(const double* x, double* y, int nrhs, cudaStream_t s, bool adj)
{
    if (nrhs <= 0) throw Error(TBEM_ERR_ARG, "n_rhs must be > 0");
    if (opt.host_only) throw Error(TBEM_ERR_STATE, "operator was built with host_only");
    DeviceGuard guard(opt.device);
    if (!s) s = stream;
    const long n_in = adj ? (long)R * n_obs : (long)R * n_src;
    const long n_out = adj ? (long)R * n_src : (long)R * n_obs;
    if (n_out == 0) return;
    cudaPointerAttributes ax{}, ay{};
    bool x_dev = x && cudaPointerGetAttributes(&ax, x) == cudaSuccess &&
                 (ax.type == cudaMemoryTypeDevice || ax.type == cudaMemoryTypeManaged);
    bool y_dev = y && cudaPointerGetAttributes(&ay, y) == cudaSuccess &&
                 (ay.type == cudaMemoryTypeDevice || ay.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    if (n_in == 0) {
        if (y_dev) TBEM_CK(cudaMemsetAsync(y, 0, sizeof(double) * n_out * nrhs, s));
        else std::memset(y, 0, sizeof(double) * n_out * nrhs);
        if (y_dev) TBEM_CK(cudaStreamSynchronize(s));
        return;
    }
    if (flags_raised())  // raised by an earlier apply
        throw Error(TBEM_ERR_TIMEOUT, "a bounded device wait of an apply gave up");
    // the right-hand sides run in chunks whose work buffers stay within a
    // fixed budget (the cell buffers grow with cells x right-hand sides)
    const int chunk = rhs_chunk(nrhs);
    io_x.ensure((size_t)n_in * nrhs);
    io_y.ensure((size_t)n_out * nrhs);
    ensure_rhs(chunk);
    launches = 0;
    mark("apply", s);  // phase means are per apply, whatever the right-hand-side chunks
    TBEM_CK(cudaMemcpyAsync(io_x.p, x, sizeof(double) * n_in * nrhs,
                            x_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    for (int r0 = 0; r0 < nrhs; r0 += chunk) {
        const int nr = std::min(chunk, nrhs - r0);
        xin = io_x.p + (long)r0 * n_in;
        yout = io_y.p + (long)r0 * n_out;
        if (adj) adjoint(nr, s);
        else forward(nr, s);
    }
    TBEM_CK(cudaMemcpyAsync(y, io_y.p, sizeof(double) * n_out * nrhs,
                            y_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    check_tc_flags(!y_dev, s);
}

// Right-hand sides per pass: as many as keep the per-right-hand-side work
// buffers (cell states, their tensor-core planes, point strengths and
// outputs) within RHS_WORK_BUDGET bytes; at least one.
int Plan::rhs_chunk(int nrhs) const
{
    constexpr double RHS_WORK_BUDGET = 24.0 * (1L << 30);
    const double ncs = (double)stree->cells.size(), nco = (double)otree.cells.size();
    const double N = (double)std::max(n_obs, n_src);
    double per = 8.0 * R * N * 4;  // io copies, strengths, outputs
    if (f.f64) {
        per += 8.0 * (ncs * n + ncs * f.r_in + nco * f.r_out);
        if (!L.p2l.empty()) per += 8.0 * nco * n;
        if (!L.m2p.empty()) per += 8.0 * ncs * n;
    } else if (f.mixed) {
        per += 4.0 * (ncs + nco) * n;
        if (f.m2l_compressed) per += 4.0 * (ncs * f.r_in + nco * f.r_out) + 6.0 * std::max(ncs, nco) * 128;
        if (!L.m2p.empty() || f.m2l_on_the_fly) per += 8.0 * (2 * ncs + nco) * n;
    } else {
        per += 8.0 * 2 * (ncs + nco) * n;
        per += 8.0 * std::max(f.m2l_slots.max_slots, f.m2l_t_slots.max_slots) * n;
    }
    return (int)std::max<double>(1.0, std::min<double>(nrhs, std::floor(RHS_WORK_BUDGET / per)));
}

// Copies the tensor-core timeout flags into pinned memory on stream s and,
// when wait_device, waits for them (host outputs: the apply is synchronous
// anyway); otherwise the copy is read by the next call.  A raised flag stays
// raised: the operator reports TBEM_ERR_TIMEOUT from then on.
void Plan::check_tc_flags(bool wait_device, cudaStream_t s)
{
    const std::vector<const int*> flags = device_flags();
    if (flags.empty()) {
        if (wait_device) TBEM_CK(cudaStreamSynchronize(s));
        return;
    }
    if (!h_err) {
        TBEM_CK(cudaMallocHost(&h_err, N_ERR_FLAGS * sizeof(int)));
        for (int i = 0; i < N_ERR_FLAGS; i++) h_err[i] = 0;
    }
    if (flags_raised()) throw Error(TBEM_ERR_TIMEOUT, "a bounded device wait of an apply gave up");
    for (size_t i = 0; i < flags.size(); i++)
        TBEM_CK(cudaMemcpyAsync(h_err + i, flags[i], sizeof(int), cudaMemcpyDeviceToHost, s));
    if (wait_device) {
        TBEM_CK(cudaStreamSynchronize(s));
        if (flags_raised()) throw Error(TBEM_ERR_TIMEOUT, "a bounded device wait of an apply gave up");
    }
}

// The device error flags of the bounded waits (the tensor-core GEMMs'; at
// most N_ERR_FLAGS).
std::vector<const int*> Plan::device_flags() const
{
    std::vector<const int*> v;
    if (f.tc.err.p) v.push_back(f.tc.err.p);
    if (f.tc_c.err.p) v.push_back(f.tc_c.err.p);
    return v;
}

bool Plan::flags_raised() const
{
    if (!h_err) return false;
    for (int i = 0; i < N_ERR_FLAGS; i++)
        if (h_err[i]) return true;
    return false;
}

void Plan::sync(cudaStream_t s)
{
    if (opt.host_only) return;
    DeviceGuard guard(opt.device);
    if (s) TBEM_CK(cudaStreamSynchronize(s));
    TBEM_CK(cudaStreamSynchronize(stream));
    TBEM_CK(cudaStreamSynchronize(side));
    const std::vector<const int*> flags = device_flags();
    bool raised = flags_raised();
    for (size_t i = 0; i < flags.size(); i++) {
        int v = 0;
        TBEM_CK(cudaMemcpy(&v, flags[i], sizeof(int), cudaMemcpyDeviceToHost));
        if (v) {
            raised = true;
            if (h_err) h_err[i] = 1;
        }
    }
    if (raised) throw Error(TBEM_ERR_TIMEOUT, "a bounded device wait of an apply gave up");
}

}  // namespace tbem
