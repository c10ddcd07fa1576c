// Obs-owner N-body evaluation: the device form of the reference's
// nbody_eval (cpp/nbody_operator.h:117-141) as it is called by P2P, P2M,
// P2L, M2P, L2P (and M2M/L2L/M2L when they are evaluated on the fly),
// cpp/fmm.cpp:163-441.
//
// A task = one target block (a range of permuted points, or the translation
// surface of one cell) plus a list of source blocks (point ranges or cell
// surfaces with densities).  One CTA owns a chunk of (128 / TPT) targets of
// one task, so every output is written by exactly one thread: no atomics and
// a fixed summation order.  TPT threads share a target and split its
// sources; their partial sums meet in a warp-shuffle reduction.  Sources are
// staged through shared memory in tiles of 128 that run across source-block
// boundaries (each source's position, normal and densities stored as
// 4-vectors, one shared load each in the pair loop).  Coordinates are
// shifted to the task's origin (the target
// cell's centre) in FP64 before the pair arithmetic, so the FP32 variant
// keeps full relative accuracy in the separations.  The FP32 variant sums
// each tile in FP32 and folds the tile sums into a compensated (Kahan) pair.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"

namespace tbem {

constexpr int EVAL_THREADS = 128;

template <typename T>
struct EvalArgs {
    // work items: CTA b handles task item_task[b], targets from item_start[b]
    const int* item_task;
    const int* item_start;
    // tasks
    const long* task_tgt;        // target block: first point, or cell id for surfaces
    const int* task_tgt_count;   // number of targets
    const double* task_origin;   // [ntask][3]
    const int* task_src_ptr;     // CSR into the source-block arrays
    const long* src_blk;         // first point, or cell id for surfaces
    const int* src_blk_count;
    const int* src_blk_prefix;   // sources before this block within its task
    const int* src_blk_near;     // per source block: 1 when its cell touches the target leaf
                                 // (point-to-point sets only; may be null)
    // target geometry
    const double* t_xyz;         // [N][3] permuted points (point targets)
    const T* t_nrm;              // [N][3]
    const double* t_center;      // [cells][3] (surface targets)
    const double* t_rad;         // [cells] |half width|
    double t_rref;
    // source geometry and strengths
    const double* s_xyz;
    const T* s_nrm;
    const double* s_nrm64;       // FP64 source normals (the double-float n . d)
    const T* s_str;              // point strengths [rhs][C][N] (weights applied)
    long s_n;                    // N (component stride); rhs stride = C * N
    const double* s_center;
    const double* s_rad;
    double s_rref;
    const T* q;                  // surface densities [cell][rhs][C * ns]
    const double* unit;          // [ns][3] unit sphere points (also the normals)
    int ns;
    // outputs
    double* y;                   // point outputs [rhs][R][y_n]
    long y_n;
    T* c;                        // surface outputs [cell][rhs][R * ns]
    int nrhs;                    // total right-hand sides (buffer strides)
    int rhs0;                    // first rhs handled by this launch
    int add;                     // 0: store, 1: add
    T c2;
    double scale;
};

// Four values of one source in shared memory, read with one vector load.
template <typename T>
struct alignas(4 * sizeof(T)) Vec4 {
    T x, y, z, w;
};

// Error-free transformation of a sum (Knuth's TwoSum): s + e = a + b exactly.
// The building block, with the FMA product error, of the compensated dot
// product of Ogita, Rump and Oishi ("Accurate sum and dot product", SIAM J.
// Sci. Comput. 26 (2005), algorithm Dot2).  The _rn intrinsics keep the
// compiler from contracting or reassociating the steps.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float z = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z));
}

// The double-layer value n . d / |d|^3 of a near pair (d = q - p) from
// positions held as hi + lo FP32 pairs (relative to the task origin) and the
// source normal as hi + lo: the separation as an unevaluated pair (TwoSum of
// the high parts, the TwoSum error and the low parts' difference folded into
// the low part), n . d by Dot2 on the high parts plus the first-order cross
// terms.  The error of n . d is a few ulps of n . d itself, where the plain
// FP32 form's is eps |d| -- for a nearly tangent pair on a curved surface
// (n . d = O(kappa h^2)) the difference between 1e-5 and 1e-7 of the pair's
// value.  Returns 0 for the self pair (|d|^2 < 1e-12).
__device__ __forceinline__ float lapd_near_df(const Vec4<float>& qh, const Vec4<float>& ql,
                                              const Vec4<float>& nh, const Vec4<float>& nl,
                                              float phx, float phy, float phz, float plx, float ply,
                                              float plz)
{
    float dh[3], dl[3];
    const float qa[3] = {qh.x, qh.y, qh.z}, qb[3] = {ql.x, ql.y, ql.z};
    const float pa[3] = {phx, phy, phz}, pb[3] = {plx, ply, plz};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float e;
        two_sum(qa[k], -pa[k], dh[k], e);
        dl[k] = __fadd_rn(e, __fsub_rn(qb[k], pb[k]));
    }
    const float dx = dh[0] + dl[0], dy = dh[1] + dl[1], dz = dh[2] + dl[2];
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < 1e-12f) return 0.f;
    const float na[3] = {nh.x, nh.y, nh.z}, nb[3] = {nl.x, nl.y, nl.z};
    float s = __fmul_rn(na[0], dh[0]);
    float c = __fmaf_rn(na[0], dh[0], -s);
#pragma unroll
    for (int k = 1; k < 3; k++) {
        const float p = __fmul_rn(na[k], dh[k]);
        const float pe = __fmaf_rn(na[k], dh[k], -p);
        float q;
        two_sum(s, p, s, q);
        c = __fadd_rn(c, __fadd_rn(q, pe));
    }
#pragma unroll
    for (int k = 0; k < 3; k++) c = __fmaf_rn(na[k], dl[k], __fmaf_rn(nb[k], dh[k], c));
    const float dn = __fadd_rn(s, c);
    const float ir = rsqrtf(r2);
    return dn * (ir * ir * ir);
}

template <typename T>
__device__ __forceinline__ void kahan_add(T& hi, T& lo, T v)
{
    T y = v - lo;
    T t = hi + y;
    lo = (t - hi) - y;
    hi = t;
}

template <int KID, bool TRANS, typename T, int NR, bool TGT_SURF, bool SRC_SURF, int TPT>
__global__ void __launch_bounds__(EVAL_THREADS)
eval_kernel(const EvalArgs<T> a)
{
    constexpr int R = kernel_dim(KID);
    constexpr int TPB = EVAL_THREADS / TPT;  // targets per CTA
    constexpr bool COMP = sizeof(T) == 4;    // compensated accumulation in FP32
    // scalar kernels with point sources and many right-hand sides: the
    // densities of four right-hand sides share one 4-vector, and the kernel
    // value is computed once per pair and applied to every right-hand side
    constexpr bool PACK = R == 1 && NR >= 4 && NR % 4 == 0 && !SRC_SURF && !TRANS;
    constexpr int NV = PACK ? NR / 4 : NR;
    // point-to-point in FP32 for a kernel with n . d: positions as hi + lo
    constexpr bool SPLIT = COMP && !SRC_SURF && !TGT_SURF && normal_dot_kernel(KID);
    // the double layer's pairs with a source block touching the target leaf:
    // double-float n . d (lapd_near_df), the block's flag in the position's w
    constexpr bool DF = SPLIT && KID == LAP_D && !TRANS;
    // per source: position, normal, and the R density components of every
    // right-hand side, each a 4-vector (one shared load in the pair loop)
    __shared__ Vec4<T> sp[EVAL_THREADS], sn[EVAL_THREADS];
    __shared__ Vec4<T> sl[SPLIT ? EVAL_THREADS : 1];  // low parts of the positions
    __shared__ Vec4<T> snl[DF ? EVAL_THREADS : 1];    // low parts of the normals
    __shared__ Vec4<T> sv[NV][EVAL_THREADS];

    const int task = a.item_task[blockIdx.x];
    const int t0 = a.item_start[blockIdx.x];
    const int ntgt = a.task_tgt_count[task];
    const int lt = threadIdx.x / TPT;
    const int lane = threadIdx.x % TPT;
    const int ti = t0 + lt;
    const bool active = lt < TPB && ti < ntgt;
    const double ox = a.task_origin[3 * task], oy = a.task_origin[3 * task + 1],
                 oz = a.task_origin[3 * task + 2];
    const long tb = a.task_tgt[task];

    // target point relative to the origin (low parts: SPLIT only)
    T px = 0, py = 0, pz = 0, pnx = 0, pny = 0, pnz = 0, plx = 0, ply = 0, plz = 0;
    if (active) {
        if (TGT_SURF) {
            const double r = a.t_rad[tb];
            const double ux = a.unit[3 * ti], uy = a.unit[3 * ti + 1], uz = a.unit[3 * ti + 2];
            px = T(r * (a.t_rref * ux) + a.t_center[3 * tb] - ox);
            py = T(r * (a.t_rref * uy) + a.t_center[3 * tb + 1] - oy);
            pz = T(r * (a.t_rref * uz) + a.t_center[3 * tb + 2] - oz);
            pnx = T(ux); pny = T(uy); pnz = T(uz);
        } else {
            const long p = tb + ti;
            const double rx = a.t_xyz[3 * p] - ox, ry = a.t_xyz[3 * p + 1] - oy,
                         rz = a.t_xyz[3 * p + 2] - oz;
            px = T(rx); py = T(ry); pz = T(rz);
            if (SPLIT) { plx = T(rx - double(px)); ply = T(ry - double(py)); plz = T(rz - double(pz)); }
            pnx = a.t_nrm[3 * p]; pny = a.t_nrm[3 * p + 1]; pnz = a.t_nrm[3 * p + 2];
        }
    }

    T acc[NR * R], lo[NR * R], part[NR * R];
#pragma unroll
    for (int i = 0; i < NR * R; i++) { acc[i] = 0; lo[i] = 0; part[i] = 0; }

    const int b0 = a.task_src_ptr[task], b1 = a.task_src_ptr[task + 1];
    const int total = b1 > b0 ? a.src_blk_prefix[b1 - 1] + a.src_blk_count[b1 - 1] : 0;
    const int nr_here = min(NR, a.nrhs - a.rhs0);
    int blk = b0;  // block containing this thread's next slot (advances monotonically)
    for (int tile = 0; tile < total; tile += EVAL_THREADS) {
        const int g = tile + threadIdx.x;
        if (g < total) {
            while (blk + 1 < b1 && a.src_blk_prefix[blk + 1] <= g) blk++;
            const int li = g - a.src_blk_prefix[blk];
            const long sb = a.src_blk[blk];
            double qx, qy, qz;
            T nx, ny, nz;
            if (SRC_SURF) {
                const double r = a.s_rad[sb];
                const double ux = a.unit[3 * li], uy = a.unit[3 * li + 1], uz = a.unit[3 * li + 2];
                qx = r * (a.s_rref * ux) + a.s_center[3 * sb];
                qy = r * (a.s_rref * uy) + a.s_center[3 * sb + 1];
                qz = r * (a.s_rref * uz) + a.s_center[3 * sb + 2];
                nx = T(ux); ny = T(uy); nz = T(uz);
                const int cn = R * a.ns;
#pragma unroll
                for (int r_ = 0; r_ < NR; r_++) {
                    T vv[3] = {T(0), T(0), T(0)};
#pragma unroll
                    for (int d = 0; d < R; d++)
                        vv[d] = r_ < nr_here ? a.q[(sb * a.nrhs + a.rhs0 + r_) * cn + d * a.ns + li] : T(0);
                    sv[r_][threadIdx.x] = Vec4<T>{vv[0], vv[1], vv[2], T(0)};
                }
            } else {
                const long p = sb + li;
                qx = a.s_xyz[3 * p]; qy = a.s_xyz[3 * p + 1]; qz = a.s_xyz[3 * p + 2];
                nx = a.s_nrm[3 * p]; ny = a.s_nrm[3 * p + 1]; nz = a.s_nrm[3 * p + 2];
                if constexpr (PACK) {
#pragma unroll
                    for (int r4 = 0; r4 < NV; r4++) {
                        T vv[4];
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const int r_ = 4 * r4 + k;
                            vv[k] = r_ < nr_here ? a.s_str[(long)(a.rhs0 + r_) * a.s_n + p] : T(0);
                        }
                        sv[r4][threadIdx.x] = Vec4<T>{vv[0], vv[1], vv[2], vv[3]};
                    }
                } else {
#pragma unroll
                    for (int r_ = 0; r_ < NR; r_++) {
                        T vv[3] = {T(0), T(0), T(0)};
#pragma unroll
                        for (int d = 0; d < R; d++)
                            vv[d] = r_ < nr_here ? a.s_str[((long)(a.rhs0 + r_) * R + d) * a.s_n + p] : T(0);
                        sv[r_][threadIdx.x] = Vec4<T>{vv[0], vv[1], vv[2], T(0)};
                    }
                }
            }
            const double rx = qx - ox, ry = qy - oy, rz = qz - oz;
            const bool near = DF && a.src_blk_near && a.src_blk_near[blk];
            const Vec4<T> hi{T(rx), T(ry), T(rz), near ? T(1) : T(0)};
            sp[threadIdx.x] = hi;
            if (SPLIT)
                sl[threadIdx.x] = Vec4<T>{T(rx - double(hi.x)), T(ry - double(hi.y)), T(rz - double(hi.z)), T(0)};
            if (near) {
                const long p = sb + li;
                const double mx = a.s_nrm64[3 * p], my = a.s_nrm64[3 * p + 1], mz = a.s_nrm64[3 * p + 2];
                nx = T(mx); ny = T(my); nz = T(mz);
                snl[threadIdx.x] = Vec4<T>{T(mx - double(nx)), T(my - double(ny)), T(mz - double(nz)), T(0)};
            }
            sn[threadIdx.x] = Vec4<T>{nx, ny, nz, T(0)};
        }
        __syncthreads();
        if (active) {
            const int n_here = min(EVAL_THREADS, total - tile);
            for (int j = lane; j < n_here; j += TPT) {
                const Vec4<T> q = sp[j];
                if constexpr (DF) {
                    if (q.w != T(0)) {
                        const T kv = lapd_near_df(q, sl[j], sn[j], snl[j], px, py, pz, plx, ply, plz);
#pragma unroll
                        for (int r4 = 0; r4 < NV; r4++) {
                            const Vec4<T> vq = sv[r4][j];
                            if constexpr (PACK) {
                                part[4 * r4] += kv * vq.x;
                                part[4 * r4 + 1] += kv * vq.y;
                                part[4 * r4 + 2] += kv * vq.z;
                                part[4 * r4 + 3] += kv * vq.w;
                            } else {
                                part[r4] += kv * vq.x;  // R = 1: one density per right-hand side
                            }
                        }
                        continue;
                    }
                }
                T dx = q.x - px, dy = q.y - py, dz = q.z - pz;
                if (SPLIT) {
                    // (q_hi - p_hi) + (q_lo - p_lo): rounding errors O(eps |d|)
                    const Vec4<T> ql = sl[j];
                    dx += ql.x - plx; dy += ql.y - ply; dz += ql.z - plz;
                }
                const Vec4<T> nq = sn[j];
                if constexpr (PACK) {
                    // the kernel value once (accumulate with a unit density)
                    T kv = 0;
                    const T one[3] = {T(1), T(0), T(0)};
                    accumulate<KID, false, T>(dx, dy, dz, pnx, pny, pnz, nq.x, nq.y, nq.z, a.c2, one, &kv);
#pragma unroll
                    for (int r4 = 0; r4 < NV; r4++) {
                        const Vec4<T> vq = sv[r4][j];
                        part[4 * r4] += kv * vq.x;
                        part[4 * r4 + 1] += kv * vq.y;
                        part[4 * r4 + 2] += kv * vq.z;
                        part[4 * r4 + 3] += kv * vq.w;
                    }
                    continue;
                }
#pragma unroll
                for (int r_ = 0; r_ < NR; r_++) {
                    const Vec4<T> vq = sv[r_][j];
                    const T v[3] = {vq.x, vq.y, vq.z};
                    // transposed apply: the target is the forward source and
                    // the source the forward observer, so the separation
                    // (forward src - forward obs) flips sign and the normals swap
                    if (TRANS)
                        accumulate<KID, true, T>(-dx, -dy, -dz, nq.x, nq.y, nq.z, pnx, pny, pnz,
                                                 a.c2, v, &part[r_ * R]);
                    else
                        accumulate<KID, false, T>(dx, dy, dz, pnx, pny, pnz, nq.x, nq.y, nq.z,
                                                  a.c2, v, &part[r_ * R]);
                }
            }
            if (COMP) {
#pragma unroll
                for (int i = 0; i < NR * R; i++) { kahan_add(acc[i], lo[i], part[i]); part[i] = 0; }
            }
        }
        __syncthreads();
    }
    if (!COMP) {
#pragma unroll
        for (int i = 0; i < NR * R; i++) acc[i] = part[i];
    }
    // reduce the TPT partial sums of a target (consecutive lanes of one warp)
#pragma unroll
    for (int off = TPT / 2; off > 0; off /= 2) {
#pragma unroll
        for (int i = 0; i < NR * R; i++) {
            T o = __shfl_xor_sync(0xffffffffu, acc[i], off);
            if (COMP) {
                // a pair (hi, lo) stands for hi - lo
                T ol = __shfl_xor_sync(0xffffffffu, lo[i], off);
                kahan_add(acc[i], lo[i], o);
                lo[i] += ol;
            } else {
                acc[i] += o;
            }
        }
    }
    if (!active || lane != 0) return;
    if (TGT_SURF) {
        const int cn = R * a.ns;
#pragma unroll
        for (int r_ = 0; r_ < NR; r_++) {
            if (r_ >= nr_here) break;
#pragma unroll
            for (int d = 0; d < R; d++) {
                T val = T(a.scale) * (acc[r_ * R + d] - (COMP ? lo[r_ * R + d] : T(0)));
                T* dst = &a.c[(tb * a.nrhs + a.rhs0 + r_) * cn + d * a.ns + ti];
                *dst = a.add ? *dst + val : val;
            }
        }
    } else {
        const long p = tb + ti;
#pragma unroll
        for (int r_ = 0; r_ < NR; r_++) {
            if (r_ >= nr_here) break;
#pragma unroll
            for (int d = 0; d < R; d++) {
                double val = a.scale * ((double)acc[r_ * R + d] - (COMP ? (double)lo[r_ * R + d] : 0.0));
                double* dst = &a.y[((long)(a.rhs0 + r_) * R + d) * a.y_n + p];
                *dst = a.add ? *dst + val : val;
            }
        }
    }
}

// Scalar 3D kernels in FP32, point sources, not transposed, WIDE right-hand
// sides per launch: the many-right-hand-side point-to-point and points-to-
// check-surface passes.  The work items are those of eval_kernel (TPB =
// 128 / TPT targets per CTA), run by half as many threads: every thread owns
// two targets (t and t + TPB / 2), so each source read from shared memory --
// position, normal and the densities of all WIDE right-hand sides, packed
// four to a 4-vector -- serves two targets, and each kernel value is applied
// to all right-hand sides.  Sums as in eval_kernel (per tile in FP32, folded
// into a compensated pair; TPT partial sums met by warp shuffles).
template <int KID, bool TGT_SURF, int TPT, int WIDE>
__global__ void __launch_bounds__(EVAL_THREADS / 2)
eval_wide_kernel(const EvalArgs<float> a)
{
    static_assert(kernel_dim(KID) == 1 && WIDE % 4 == 0, "scalar kernels, packed right-hand sides");
    constexpr int NT = EVAL_THREADS / 2;     // threads of the CTA
    constexpr int NV = WIDE / 4;             // 4-vectors of densities per source
    constexpr int TPB = EVAL_THREADS / TPT;  // targets per CTA (as the items were cut)
    constexpr int HALF = TPB / 2;            // a thread's second target is HALF further
    constexpr bool SPLIT = !TGT_SURF && normal_dot_kernel(KID);  // positions as hi + lo
    // the double layer's pairs with a source block touching the target leaf
    // take the double-float n . d (lapd_near_df; the block's flag rides in
    // the position's w); the source normals' low parts are staged for them
    constexpr bool DF = SPLIT && KID == LAP_D;
    __shared__ Vec4<float> sp[EVAL_THREADS], sn[EVAL_THREADS];
    __shared__ Vec4<float> sl[SPLIT ? EVAL_THREADS : 1];
    __shared__ Vec4<float> snl[DF ? EVAL_THREADS : 1];
    __shared__ Vec4<float> sv[NV][EVAL_THREADS];

    const int task = a.item_task[blockIdx.x];
    const int t0 = a.item_start[blockIdx.x];
    const int ntgt = a.task_tgt_count[task];
    const int lt = threadIdx.x / TPT;  // < HALF
    const int lane = threadIdx.x % TPT;
    const double ox = a.task_origin[3 * task], oy = a.task_origin[3 * task + 1],
                 oz = a.task_origin[3 * task + 2];
    const long tb = a.task_tgt[task];

    float px[2], py[2], pz[2], pnx[2], pny[2], pnz[2], plx[2], ply[2], plz[2];
    bool act[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int ti = t0 + lt + q * HALF;
        act[q] = ti < ntgt;
        px[q] = py[q] = pz[q] = pnx[q] = pny[q] = pnz[q] = 0.f;
        plx[q] = ply[q] = plz[q] = 0.f;
        if (!act[q]) continue;
        if (TGT_SURF) {
            const double r = a.t_rad[tb];
            const double ux = a.unit[3 * ti], uy = a.unit[3 * ti + 1], uz = a.unit[3 * ti + 2];
            px[q] = float(r * (a.t_rref * ux) + a.t_center[3 * tb] - ox);
            py[q] = float(r * (a.t_rref * uy) + a.t_center[3 * tb + 1] - oy);
            pz[q] = float(r * (a.t_rref * uz) + a.t_center[3 * tb + 2] - oz);
            pnx[q] = float(ux); pny[q] = float(uy); pnz[q] = float(uz);
        } else {
            const long p = tb + ti;
            const double rx = a.t_xyz[3 * p] - ox, ry = a.t_xyz[3 * p + 1] - oy,
                         rz = a.t_xyz[3 * p + 2] - oz;
            px[q] = float(rx); py[q] = float(ry); pz[q] = float(rz);
            if (SPLIT) {
                plx[q] = float(rx - double(px[q]));
                ply[q] = float(ry - double(py[q]));
                plz[q] = float(rz - double(pz[q]));
            }
            pnx[q] = a.t_nrm[3 * p]; pny[q] = a.t_nrm[3 * p + 1]; pnz[q] = a.t_nrm[3 * p + 2];
        }
    }

    float acc[2][WIDE], lo[2][WIDE], part[2][WIDE];
#pragma unroll
    for (int q = 0; q < 2; q++)
#pragma unroll
        for (int i = 0; i < WIDE; i++) { acc[q][i] = 0.f; lo[q][i] = 0.f; part[q][i] = 0.f; }

    const int b0 = a.task_src_ptr[task], b1 = a.task_src_ptr[task + 1];
    const int total = b1 > b0 ? a.src_blk_prefix[b1 - 1] + a.src_blk_count[b1 - 1] : 0;
    const int nr_here = min(WIDE, a.nrhs - a.rhs0);
    int blk = b0;  // advances monotonically: a thread's slots only grow
    for (int tile = 0; tile < total; tile += EVAL_THREADS) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int slot = threadIdx.x + h * NT;
            const int g = tile + slot;
            if (g >= total) continue;
            while (blk + 1 < b1 && a.src_blk_prefix[blk + 1] <= g) blk++;
            const long p = a.src_blk[blk] + (g - a.src_blk_prefix[blk]);
            const double rx = a.s_xyz[3 * p] - ox, ry = a.s_xyz[3 * p + 1] - oy,
                         rz = a.s_xyz[3 * p + 2] - oz;
            const bool near = DF && a.src_blk_near && a.src_blk_near[blk];
            const Vec4<float> hi{float(rx), float(ry), float(rz), near ? 1.f : 0.f};
            sp[slot] = hi;
            if (SPLIT)
                sl[slot] = Vec4<float>{float(rx - double(hi.x)), float(ry - double(hi.y)),
                                       float(rz - double(hi.z)), 0.f};
            if (near) {
                const double nx = a.s_nrm64[3 * p], ny = a.s_nrm64[3 * p + 1], nz = a.s_nrm64[3 * p + 2];
                const Vec4<float> nh{float(nx), float(ny), float(nz), 0.f};
                sn[slot] = nh;
                snl[slot] = Vec4<float>{float(nx - double(nh.x)), float(ny - double(nh.y)),
                                        float(nz - double(nh.z)), 0.f};
            } else {
                sn[slot] = Vec4<float>{a.s_nrm[3 * p], a.s_nrm[3 * p + 1], a.s_nrm[3 * p + 2], 0.f};
            }
#pragma unroll
            for (int r4 = 0; r4 < NV; r4++) {
                float vv[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int r_ = 4 * r4 + k;
                    vv[k] = r_ < nr_here ? a.s_str[(long)(a.rhs0 + r_) * a.s_n + p] : 0.f;
                }
                sv[r4][slot] = Vec4<float>{vv[0], vv[1], vv[2], vv[3]};
            }
        }
        __syncthreads();
        if (act[0] || act[1]) {
            const int n_here = min(EVAL_THREADS, total - tile);
            const float one[3] = {1.f, 0.f, 0.f};
            for (int j = lane; j < n_here; j += TPT) {
                const Vec4<float> s = sp[j];
                const Vec4<float> nq = sn[j];
                const Vec4<float> sq = SPLIT ? sl[j] : Vec4<float>{0.f, 0.f, 0.f, 0.f};
                float kv[2] = {0.f, 0.f};
                if (DF && s.w != 0.f) {
                    const Vec4<float> nl = snl[j];
#pragma unroll
                    for (int q = 0; q < 2; q++)
                        kv[q] = lapd_near_df(s, sq, nq, nl, px[q], py[q], pz[q], plx[q], ply[q], plz[q]);
                } else {
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        float dx = s.x - px[q], dy = s.y - py[q], dz = s.z - pz[q];
                        if (SPLIT) { dx += sq.x - plx[q]; dy += sq.y - ply[q]; dz += sq.z - plz[q]; }
                        accumulate<KID, false, float>(dx, dy, dz, pnx[q], pny[q], pnz[q], nq.x, nq.y,
                                                      nq.z, a.c2, one, &kv[q]);
                    }
                }
#pragma unroll
                for (int r4 = 0; r4 < NV; r4++) {
                    const Vec4<float> vq = sv[r4][j];
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        part[q][4 * r4] += kv[q] * vq.x;
                        part[q][4 * r4 + 1] += kv[q] * vq.y;
                        part[q][4 * r4 + 2] += kv[q] * vq.z;
                        part[q][4 * r4 + 3] += kv[q] * vq.w;
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 2; q++)
#pragma unroll
                for (int i = 0; i < WIDE; i++) { kahan_add(acc[q][i], lo[q][i], part[q][i]); part[q][i] = 0.f; }
        }
        __syncthreads();
    }
    // the TPT partial sums of a target pair (consecutive lanes of one warp)
#pragma unroll
    for (int off = TPT / 2; off > 0; off /= 2) {
#pragma unroll
        for (int q = 0; q < 2; q++)
#pragma unroll
            for (int i = 0; i < WIDE; i++) {
                const float o = __shfl_xor_sync(0xffffffffu, acc[q][i], off);
                const float ol = __shfl_xor_sync(0xffffffffu, lo[q][i], off);
                kahan_add(acc[q][i], lo[q][i], o);
                lo[q][i] += ol;
            }
    }
    if (lane != 0) return;
#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (!act[q]) continue;
        const int ti = t0 + lt + q * HALF;
#pragma unroll
        for (int r_ = 0; r_ < WIDE; r_++) {
            if (r_ >= nr_here) break;
            if (TGT_SURF) {
                const float val = float(a.scale) * (acc[q][r_] - lo[q][r_]);
                float* dst = &a.c[(tb * a.nrhs + a.rhs0 + r_) * (long)a.ns + ti];
                *dst = a.add ? *dst + val : val;
            } else {
                const double val = a.scale * ((double)acc[q][r_] - (double)lo[q][r_]);
                double* dst = &a.y[(long)(a.rhs0 + r_) * a.y_n + tb + ti];
                *dst = a.add ? *dst + val : val;
            }
        }
    }
}

}  // namespace tbem
