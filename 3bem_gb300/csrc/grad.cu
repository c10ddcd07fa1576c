// Kernel-gradient pass: derivatives of  L = r^T A x,  A_ij = w_j K(x_i, y_j; n_i, n_j),
// with respect to every point position, normal and weight, and to x (the
// direct operator's transpose apply), in FP64.
//
// The kernel tensors are differentiated exactly by forward-mode dual numbers:
// kernel_tensor<T> (kernels.cuh) is evaluated with T = Dual<3> seeded on the
// separation delta = y - x (d/dy = d/ddelta, d/dx = -d/ddelta), on the source
// normal, or on the observation normal.  Two passes, each owning its outputs
// (no atomics): a source-owner pass (gradients of y_j, n_j, w_j and x_j) and
// an observation-owner pass (gradients of x_i and n_i).  Direct O(N M) sums:
// the workload this serves (24,576 sources x 16,384 observers) takes a
// fraction of a second.
#include <string>

#include "plan.h"

namespace tbem {
namespace {

struct Dual3 {
    double v, g[3];
    __device__ Dual3() : v(0), g{0, 0, 0} {}
    __device__ Dual3(double x) : v(x), g{0, 0, 0} {}
};
__device__ __forceinline__ Dual3 operator+(const Dual3& a, const Dual3& b)
{
    Dual3 r; r.v = a.v + b.v;
    for (int k = 0; k < 3; k++) r.g[k] = a.g[k] + b.g[k];
    return r;
}
__device__ __forceinline__ Dual3 operator-(const Dual3& a, const Dual3& b)
{
    Dual3 r; r.v = a.v - b.v;
    for (int k = 0; k < 3; k++) r.g[k] = a.g[k] - b.g[k];
    return r;
}
__device__ __forceinline__ Dual3 operator-(const Dual3& a)
{
    Dual3 r; r.v = -a.v;
    for (int k = 0; k < 3; k++) r.g[k] = -a.g[k];
    return r;
}
__device__ __forceinline__ Dual3 operator*(const Dual3& a, const Dual3& b)
{
    Dual3 r; r.v = a.v * b.v;
    for (int k = 0; k < 3; k++) r.g[k] = a.g[k] * b.v + a.v * b.g[k];
    return r;
}
__device__ __forceinline__ Dual3 operator/(const Dual3& a, const Dual3& b)
{
    Dual3 r; r.v = a.v / b.v;
    const double ib = 1.0 / b.v;
    for (int k = 0; k < 3; k++) r.g[k] = (a.g[k] - r.v * b.g[k]) * ib;
    return r;
}
__device__ __forceinline__ bool operator<(const Dual3& a, const Dual3& b) { return a.v < b.v; }
__device__ __forceinline__ Dual3 sqrt(const Dual3& a)
{
    Dual3 r; r.v = ::sqrt(a.v);
    const double h = r.v > 0 ? 0.5 / r.v : 0.0;
    for (int k = 0; k < 3; k++) r.g[k] = a.g[k] * h;
    return r;
}

// which: 0 seeds delta, 1 the source normal, 2 the observation normal
__device__ __forceinline__ Dual3 contraction(int kid, int which, const double* d, const double* no,
                                            const double* ns, const double* rv, const double* xv,
                                            const KParams& p)
{
    Dual3 D[3], NO[3], NS[3];
    for (int k = 0; k < 3; k++) {
        D[k] = Dual3(d[k]);
        NO[k] = Dual3(no[k]);
        NS[k] = Dual3(ns[k]);
    }
    Dual3* seed = which == 0 ? D : which == 1 ? NS : NO;
    for (int k = 0; k < 3; k++) seed[k].g[k] = 1.0;
    Dual3 K[9];
    kernel_tensor<Dual3>(kid, D[0], D[1], D[2], NO[0], NO[1], NO[2], NS[0], NS[1], NS[2], p, K);
    const int R = kernel_dim(kid);
    Dual3 c(0.0);
    for (int a = 0; a < R; a++)
        for (int b = 0; b < R; b++) c = c + K[a * R + b] * Dual3(rv[a] * xv[b]);
    return c;
}

// Source owner: g_y, g_ns, g_w, g_x (= A^T r) for source j.
__global__ void grad_src_kernel(int kid, KParams p, const double* ox, const double* on, long n_obs,
                                const double* sx, const double* sn, const double* sw, long n_src,
                                const double* x, const double* r, double* g_y, double* g_ns,
                                double* g_w, double* g_x)
{
    const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_src) return;
    const int R = kernel_dim(kid);
    const bool use_ns = kid == LAP_D || kid == EL_TRAC || kid == EL_HYP;
    double xv[3] = {0, 0, 0};
    for (int b = 0; b < R; b++) xv[b] = x[b * n_src + j];
    const double y[3] = {sx[3 * j], sx[3 * j + 1], sx[3 * j + 2]};
    const double nsj[3] = {sn[3 * j], sn[3 * j + 1], sn[3 * j + 2]};
    double gy[3] = {0, 0, 0}, gn[3] = {0, 0, 0}, gw = 0, gx[3] = {0, 0, 0};
    for (long i = 0; i < n_obs; i++) {
        const double d[3] = {y[0] - ox[3 * i], y[1] - ox[3 * i + 1], y[2] - ox[3 * i + 2]};
        const double noi[3] = {on[3 * i], on[3 * i + 1], on[3 * i + 2]};
        double rv[3] = {0, 0, 0};
        for (int a = 0; a < R; a++) rv[a] = r[a * n_obs + i];
        const Dual3 c = contraction(kid, 0, d, noi, nsj, rv, xv, p);
        gw += c.v;
        for (int k = 0; k < 3; k++) gy[k] += c.g[k];
        if (use_ns) {
            const Dual3 cn = contraction(kid, 1, d, noi, nsj, rv, xv, p);
            for (int k = 0; k < 3; k++) gn[k] += cn.g[k];
        }
        // x gradient: sum_a r_a K_ab, i.e. the contraction with x = e_b
        double K[9];
        kernel_tensor<double>(kid, d[0], d[1], d[2], noi[0], noi[1], noi[2], nsj[0], nsj[1], nsj[2], p, K);
        for (int b = 0; b < R; b++)
            for (int a = 0; a < R; a++) gx[b] += rv[a] * K[a * R + b];
    }
    const double w = sw[j];
    for (int k = 0; k < 3; k++) {
        if (g_y) g_y[3 * j + k] = w * gy[k];
        if (g_ns) g_ns[3 * j + k] = w * gn[k];
    }
    if (g_w) g_w[j] = gw;
    if (g_x)
        for (int b = 0; b < R; b++) g_x[b * n_src + j] = w * gx[b];
}

// Observation owner: g_x_obs (= -dL/ddelta summed) and g_no for observer i.
__global__ void grad_obs_kernel(int kid, KParams p, const double* ox, const double* on, long n_obs,
                                const double* sx, const double* sn, const double* sw, long n_src,
                                const double* x, const double* r, double* g_o, double* g_no)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_obs) return;
    const int R = kernel_dim(kid);
    const bool use_no = kid == EL_ADJ || kid == EL_HYP;
    double rv[3] = {0, 0, 0};
    for (int a = 0; a < R; a++) rv[a] = r[a * n_obs + i];
    const double o[3] = {ox[3 * i], ox[3 * i + 1], ox[3 * i + 2]};
    const double noi[3] = {on[3 * i], on[3 * i + 1], on[3 * i + 2]};
    double go[3] = {0, 0, 0}, gn[3] = {0, 0, 0};
    for (long j = 0; j < n_src; j++) {
        const double d[3] = {sx[3 * j] - o[0], sx[3 * j + 1] - o[1], sx[3 * j + 2] - o[2]};
        const double nsj[3] = {sn[3 * j], sn[3 * j + 1], sn[3 * j + 2]};
        double xv[3] = {0, 0, 0};
        for (int b = 0; b < R; b++) xv[b] = sw[j] * x[b * n_src + j];
        const Dual3 c = contraction(kid, 0, d, noi, nsj, rv, xv, p);
        for (int k = 0; k < 3; k++) go[k] -= c.g[k];
        if (use_no) {
            const Dual3 cn = contraction(kid, 2, d, noi, nsj, rv, xv, p);
            for (int k = 0; k < 3; k++) gn[k] += cn.g[k];
        }
    }
    for (int k = 0; k < 3; k++) {
        if (g_o) g_o[3 * i + k] = go[k];
        if (g_no) g_no[3 * i + k] = gn[k];
    }
}

// Source-side gradients through the FMM's transposed passes.  For every
// source point j (a target here) and every source z of one transposed pass
// -- an observation point with density r (P2P^T), or a point of a check
// surface with the transposed state as its density (P2M^T, P2L^T) -- the
// contraction c = v(z)^T K(y_j - z; n_z, n_j) x_j, its gradient in y_j and
// (kernels with a source normal) in n_j are summed; the sums of c are
// dL/dw_j.  GRAD_TPT threads per target split its sources and meet in warp
// shuffles; the work items are those of the transposed task sets (32
// targets per CTA of 128 threads).
struct GradEvalArgs {
    const int* item_task;
    const int* item_start;
    const long* task_tgt;
    const int* task_tgt_count;
    const int* task_src_ptr;
    const long* src_blk;
    const int* src_blk_count;
    const double* t_xyz;   // source points, tree order [n][3]
    const double* t_nrm;
    const double* t_x;     // their densities x, tree order [R][t_n]
    long t_n;
    const double* s_xyz;   // point sources (observation points, tree order)
    const double* s_nrm;
    const double* s_v;     // their densities r [R][s_n]
    long s_n;
    const double* s_center;  // surface sources: cell centres, radii, the unit sphere
    const double* s_rad;
    double s_rref;
    const double* unit;
    int ns;
    const float* q32;      // surface densities [cell][R ns] (one right-hand side)
    const double* q64;
    int kid;
    KParams kp;
    int want_n;
    // 0: the targets are the operator's source points (contraction v^T K x_j,
    // derivatives in y_j and n_j); 1: its observation points (r_i^T K v,
    // derivatives in x_i and the observation normal n_i)
    int obs_side;
    double* g;             // [t_n][7]: d/dposition (3), d/dnormal (3), value (1); accumulated
};
constexpr int GRAD_TPT = 4, GRAD_THREADS = 128;

template <bool SRC_SURF>
__global__ void __launch_bounds__(GRAD_THREADS) grad_eval_kernel(const GradEvalArgs a)
{
    const int task = a.item_task[blockIdx.x];
    const int ti = a.item_start[blockIdx.x] + (int)threadIdx.x / GRAD_TPT;
    const int lane = threadIdx.x % GRAD_TPT;
    const bool active = ti < a.task_tgt_count[task];
    const int R = kernel_dim(a.kid);
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    if (active) {
        const long j = a.task_tgt[task] + ti;
        const double y[3] = {a.t_xyz[3 * j], a.t_xyz[3 * j + 1], a.t_xyz[3 * j + 2]};
        const double nj[3] = {a.t_nrm[3 * j], a.t_nrm[3 * j + 1], a.t_nrm[3 * j + 2]};
        double xv[3] = {0, 0, 0};
        for (int b = 0; b < R; b++) xv[b] = a.t_x[b * a.t_n + j];
        for (int blk = a.task_src_ptr[task]; blk < a.task_src_ptr[task + 1]; blk++) {
            const long sb = a.src_blk[blk];
            const int cnt = a.src_blk_count[blk];
            for (int li = lane; li < cnt; li += GRAD_TPT) {
                double z[3], nz[3], rv[3] = {0, 0, 0};
                if (SRC_SURF) {
                    const double rr = a.s_rad[sb];
                    for (int k = 0; k < 3; k++) {
                        const double u = a.unit[3 * li + k];
                        z[k] = rr * (a.s_rref * u) + a.s_center[3 * sb + k];
                        nz[k] = u;
                    }
                    const long base = sb * (long)(R * a.ns) + li;
                    for (int d = 0; d < R; d++)
                        rv[d] = a.q32 ? (double)a.q32[base + d * a.ns] : a.q64[base + d * a.ns];
                } else {
                    const long p = sb + li;
                    for (int k = 0; k < 3; k++) {
                        z[k] = a.s_xyz[3 * p + k];
                        nz[k] = a.s_nrm[3 * p + k];
                    }
                    for (int d = 0; d < R; d++) rv[d] = a.s_v[d * a.s_n + p];
                }
                if (!a.obs_side) {
                    // forward separation y_j - z, the target the source side
                    const double dd[3] = {y[0] - z[0], y[1] - z[1], y[2] - z[2]};
                    const Dual3 c = contraction(a.kid, 0, dd, nz, nj, rv, xv, a.kp);
                    acc[6] += c.v;
                    for (int k = 0; k < 3; k++) acc[k] += c.g[k];
                    if (a.want_n) {
                        const Dual3 cn = contraction(a.kid, 1, dd, nz, nj, rv, xv, a.kp);
                        for (int k = 0; k < 3; k++) acc[3 + k] += cn.g[k];
                    }
                } else {
                    // forward separation z - x_i: d/dx_i = -d/dd
                    const double dd[3] = {z[0] - y[0], z[1] - y[1], z[2] - y[2]};
                    const Dual3 c = contraction(a.kid, 0, dd, nj, nz, xv, rv, a.kp);
                    acc[6] += c.v;
                    for (int k = 0; k < 3; k++) acc[k] -= c.g[k];
                    if (a.want_n) {
                        const Dual3 cn = contraction(a.kid, 2, dd, nj, nz, xv, rv, a.kp);
                        for (int k = 0; k < 3; k++) acc[3 + k] += cn.g[k];
                    }
                }
            }
        }
    }
    for (int off = GRAD_TPT / 2; off > 0; off /= 2)
        for (int i = 0; i < 7; i++) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], off);
    if (!active || lane != 0) return;
    double* g = a.g + 7 * (a.task_tgt[task] + ti);
    for (int i = 0; i < 7; i++) g[i] += acc[i];
}

// Tree order [n][7] -> the caller's order: g_y = w dL/dy, g_n = w dL/dn,
// g_w = the value sum (any output may be null; w null: no weight).
__global__ void grad_scatter_kernel(const double* g7, const long* perm, const double* w, long n,
                                    double* g_y, double* g_n, double* g_w)
{
    for (long j = (long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long)gridDim.x * blockDim.x) {
        const long o = perm[j];
        const double wj = w ? w[j] : 1.0;
        for (int k = 0; k < 3; k++) {
            if (g_y) g_y[3 * o + k] = wj * g7[7 * j + k];
            if (g_n) g_n[3 * o + k] = wj * g7[7 * j + 3 + k];
        }
        if (g_w) g_w[o] = g7[7 * j + 6];
    }
}

bool dev_ptr(const void* p)
{
    cudaPointerAttributes a{};
    bool d = p && cudaPointerGetAttributes(&a, p) == cudaSuccess &&
             (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    return d;
}

struct In {
    DBuf<double> own;
    const double* p = nullptr;
    void stage(const double* h, size_t n, cudaStream_t s)
    {
        if (!n) return;
        if (dev_ptr(h)) { p = h; return; }
        own.alloc(n);
        TBEM_CK(cudaMemcpyAsync(own.p, h, n * sizeof(double), cudaMemcpyHostToDevice, s));
        p = own.p;
    }
};

struct Out {
    DBuf<double> own;
    double* user = nullptr;
    double* p = nullptr;
    size_t n = 0;
    void stage(double* h, size_t count)
    {
        user = h;
        n = count;
        if (!h || !count) return;
        if (dev_ptr(h)) { p = h; return; }
        own.alloc(count);
        p = own.p;
    }
    void finish(cudaStream_t s)
    {
        if (user && p && p != user)
            TBEM_CK(cudaMemcpyAsync(user, p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
};

// One transposed pass of the source gradients over a task set.
void grad_pass(const TaskSet& ts, bool src_surf, GradEvalArgs a, cudaStream_t s, long* launches)
{
    if (ts.n_items() == 0) return;
    a.item_task = ts.d_item_task.p;
    a.item_start = ts.d_item_start.p;
    a.task_tgt = ts.d_tgt.p;
    a.task_tgt_count = ts.d_tgt_count.p;
    a.task_src_ptr = ts.d_src_ptr.p;
    a.src_blk = ts.d_blk.p;
    a.src_blk_count = ts.d_blk_count.p;
    if (src_surf) grad_eval_kernel<true><<<ts.n_items(), GRAD_THREADS, 0, s>>>(a);
    else grad_eval_kernel<false><<<ts.n_items(), GRAD_THREADS, 0, s>>>(a);
    TBEM_CK(cudaGetLastError());
    if (launches) (*launches)++;
}

// [R][n] in the caller's order -> tree order, times w (tree order) when given
__global__ void gather_rows_kernel(const double* x, const long* perm, double* out, long n, int R,
                                   const double* w = nullptr)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n * R; t += (long)gridDim.x * blockDim.x) {
        const long i = t % n, d = t / n;
        out[t] = w ? w[i] * x[d * n + perm[i]] : x[d * n + perm[i]];
    }
}

__global__ void widen_kernel(const float* in, double* out, long n)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
        out[t] = (double)in[t];
}

unsigned blocks_for(long n) { return (unsigned)std::max<long>(1, std::min<long>((n + 255) / 256, 152L * 32)); }

}  // namespace

// The transposed apply of r leaves the transposed states of the source
// leaves' up-check surfaces (cu) and of the P2L cells' down-check surfaces
// (cd) in the work buffers; the three passes that reach source points
// (P2P^T, P2M^T, P2L^T) are then run again with the kernel's derivatives.
// The compressed forms only: their transposed states are check potentials
// on fixed surfaces, so every dependence on a source point's position and
// normal sits in these three passes.
void Plan::source_gradients(const double* x, const double* r, double* g_y, double* g_n,
                            double* g_w, cudaStream_t s)
{
    if (opt.host_only) throw Error(TBEM_ERR_STATE, "operator was built with host_only");
    if (sdim != 3) throw Error(TBEM_ERR_ARG, "source gradients take the 3D kernels");
    if (!batch_off.empty())
        throw Error(TBEM_ERR_STATE, "source gradients are not defined for the batched form "
                                    "(its meshes are rescaled by their own bounding boxes)");
    if (!(f.mixed && f.m2l_compressed) || f.m2l_on_the_fly)
        throw Error(TBEM_ERR_STATE, "source gradients need a compressed form (the precision or "
                                    "FP64 compressed form with compressible M2L operators)");
    if (!x || !r) throw Error(TBEM_ERR_ARG, "null input");
    DeviceGuard guard(opt.device);
    if (!s) s = stream;
    const long NS = n_src, NO = n_obs;
    if (NS == 0) return;
    // the work arrays: tree-order gradients [NS][7], x in tree order, r in
    // tree order, the transposed apply's output, the caller-order outputs
    const size_t off_x = 7 * (size_t)NS, off_r = off_x + R * (size_t)NS,
                 off_o = off_r + R * (size_t)std::max<long>(NO, 1), off_u = off_o + R * (size_t)NS,
                 total = off_u + 7 * (size_t)NS;
    grad_buf.ensure(total);
    double* g7 = grad_buf.p;
    double* xt = grad_buf.p + off_x;
    double* rt = grad_buf.p + off_r;
    double* out = grad_buf.p + off_o;
    double* gu = grad_buf.p + off_u;
    apply(r, out, 1, s, true);  // r is in io_x now, the transposed states in cu / cd
    // x to the device (io_y is free after the apply), then both to tree order
    TBEM_CK(cudaMemcpyAsync(io_y.p, x, sizeof(double) * R * NS, cudaMemcpyDefault, s));
    gather_rows_kernel<<<blocks_for(NS * R), 256, 0, s>>>(io_y.p, dsrc->perm.p, xt, NS, R);
    TBEM_CK(cudaGetLastError());
    if (NO > 0) {
        gather_rows_kernel<<<blocks_for(NO * R), 256, 0, s>>>(io_x.p, dobs.perm.p, rt, NO, R);
        TBEM_CK(cudaGetLastError());
    }
    TBEM_CK(cudaMemsetAsync(g7, 0, sizeof(double) * 7 * NS, s));
    GradEvalArgs a{};
    a.t_xyz = dsrc->xyz.p;
    a.t_nrm = dsrc->nrm64.p;
    a.t_x = xt;
    a.t_n = NS;
    a.unit = d_unit.p;
    a.ns = ns;
    a.g = g7;
    auto with_normals = [](int k) { return k == LAP_D || k == EL_TRAC || k == EL_HYP; };
    // P2P^T: the observation points with the densities r
    a.kid = kid;
    a.kp = make_kparams(kid, mu, nu);
    a.want_n = with_normals(kid);
    a.s_xyz = dobs.xyz.p;
    a.s_nrm = dobs.nrm64.p;
    a.s_v = rt;
    a.s_n = NO;
    grad_pass(p2p_t, false, a, s, &launches);
    // P2M^T and P2L^T: check surfaces with the transposed states
    a.kid = f.ks_kid;
    a.kp = make_kparams(f.ks_kid, mu, nu);
    a.want_n = with_normals(f.ks_kid);
    a.q32 = f.f64 ? nullptr : cu32.p;
    a.q64 = f.f64 ? cu64.p : nullptr;
    a.s_center = dsrc->center.p;
    a.s_rad = dsrc->rad.p;
    a.s_rref = f.r_uc;
    grad_pass(p2m_t, true, a, s, &launches);
    if (!L.p2l.empty()) {
        a.q32 = f.f64 ? nullptr : cd32.p;
        a.q64 = f.f64 ? cd64.p : nullptr;
        a.s_center = dobs.center.p;
        a.s_rad = dobs.rad.p;
        a.s_rref = f.r_dc;
        grad_pass(p2l_t, true, a, s, &launches);
    }
    // to the caller's order (device scratch, then wherever the caller's arrays are)
    grad_scatter_kernel<<<blocks_for(NS), 256, 0, s>>>(g7, dsrc->perm.p, dsrc->w.p, NS, gu, gu + 3 * NS,
                                                       gu + 6 * NS);
    TBEM_CK(cudaGetLastError());
    if (g_y) TBEM_CK(cudaMemcpyAsync(g_y, gu, sizeof(double) * 3 * NS, cudaMemcpyDefault, s));
    if (g_n) TBEM_CK(cudaMemcpyAsync(g_n, gu + 3 * NS, sizeof(double) * 3 * NS, cudaMemcpyDefault, s));
    if (g_w) TBEM_CK(cudaMemcpyAsync(g_w, gu + 6 * NS, sizeof(double) * NS, cudaMemcpyDefault, s));
    check_tc_flags(true, s);
}

// The forward apply of x leaves the downward coefficients of every cell
// (cdc) and the M2P sources' equivalent densities in the work buffers.  The
// passes that reach observation points -- P2P (the source points with
// densities w x), M2P (those densities on the sources' up-equivalent
// surfaces) and L2P (the leaves' down-equivalent densities, rebuilt here as
// C2E_down(level) V cdc, the product the leaf operators E V fold in) -- are
// run again with the kernel's derivatives in the observation point and its
// normal.  Compressed forms only, as for the source side.
void Plan::observation_gradients(const double* x, const double* r, double* g_x, double* g_n,
                                 cudaStream_t s)
{
    if (opt.host_only) throw Error(TBEM_ERR_STATE, "operator was built with host_only");
    if (sdim != 3) throw Error(TBEM_ERR_ARG, "observation gradients take the 3D kernels");
    if (!batch_off.empty())
        throw Error(TBEM_ERR_STATE, "observation gradients are not defined for the batched form "
                                    "(its meshes are rescaled by their own bounding boxes)");
    if (!(f.mixed && f.m2l_compressed) || f.m2l_on_the_fly)
        throw Error(TBEM_ERR_STATE, "observation gradients need a compressed form (the precision "
                                    "or FP64 compressed form with compressible M2L operators)");
    if (!x || !r) throw Error(TBEM_ERR_ARG, "null input");
    DeviceGuard guard(opt.device);
    if (!s) s = stream;
    const long NS = n_src, NO = n_obs;
    if (NO == 0) return;
    const Tree& O = otree;
    const long nco = (long)O.cells.size();
    // work arrays: tree-order gradients [NO][7], r and w x in tree order, the
    // forward output, the caller-order outputs, the leaves' down-check
    // potentials and down-equivalent densities (FP64, [cell][n])
    const size_t off_r = 7 * (size_t)NO, off_x = off_r + R * (size_t)NO,
                 off_o = off_x + R * (size_t)std::max<long>(NS, 1), off_u = off_o + R * (size_t)NO,
                 off_c = off_u + 6 * (size_t)NO, off_q = off_c + (size_t)nco * n,
                 total = off_q + (size_t)nco * n;
    grad_buf.ensure(total);
    double* g7 = grad_buf.p;
    double* rt = grad_buf.p + off_r;
    double* xt = grad_buf.p + off_x;
    double* out = grad_buf.p + off_o;
    double* gu = grad_buf.p + off_u;
    double* uck = grad_buf.p + off_c;
    double* qdn = grad_buf.p + off_q;
    apply(x, out, 1, s, false);  // x is in io_x now, the states in cdc / the M2P buffers
    TBEM_CK(cudaMemcpyAsync(io_y.p, r, sizeof(double) * R * NO, cudaMemcpyDefault, s));
    gather_rows_kernel<<<blocks_for(NO * R), 256, 0, s>>>(io_y.p, dobs.perm.p, rt, NO, R);
    TBEM_CK(cudaGetLastError());
    if (NS > 0) {
        gather_rows_kernel<<<blocks_for(NS * R), 256, 0, s>>>(io_x.p, dsrc->perm.p, xt, NS, R, dsrc->w.p);
        TBEM_CK(cudaGetLastError());
    }
    // down-check potentials of the L2P leaves (V cdc), then their
    // down-equivalent densities C2E_down(level) u, level by level in FP64
    TBEM_CK(cudaMemsetAsync(uck, 0, sizeof(double) * nco * n, s));
    if (f.f64) {
        f.decomp_l2p.run_rect<double>(cdc64.p, uck, n, f.r_out, f.r_out, 1, 0, GEMM_STORE, s, &launches);
    } else {
        TBEM_CK(cudaMemsetAsync(cd32.p, 0, sizeof(float) * nco * n, s));
        f.decomp_l2p.run_rect<float>(cdc32.p, cd32.p, n, f.r_out, f.r_out, 1, 0, GEMM_STORE, s, &launches);
        widen_kernel<<<blocks_for(nco * n), 256, 0, s>>>(cd32.p, uck, nco * n);
        TBEM_CK(cudaGetLastError());
    }
    TBEM_CKB(cublasSetStream(cublas, s));
    const double one = 1.0, zero = 0.0;
    for (int l = 0; l < O.n_levels() && l < (int)f.c2e_dn_off.size(); l++) {
        const long c0 = O.level_start[l], c1 = O.level_start[l + 1];
        if (c1 <= c0) continue;
        // column-major q (n x cells) = C2E^T-as-stored^T u: the row-major
        // pseudo-inverse applied to every cell's potential
        TBEM_CKB(cublasDgemm(cublas, CUBLAS_OP_T, CUBLAS_OP_N, n, (int)(c1 - c0), n, &one,
                             f.c2e.p + f.c2e_dn_off[l], n, uck + c0 * n, n, &zero, qdn + c0 * n, n));
    }
    TBEM_CKB(cublasSetStream(cublas, stream));
    TBEM_CK(cudaMemsetAsync(g7, 0, sizeof(double) * 7 * NO, s));
    GradEvalArgs a{};
    a.obs_side = 1;
    a.t_xyz = dobs.xyz.p;
    a.t_nrm = dobs.nrm64.p;
    a.t_x = rt;
    a.t_n = NO;
    a.unit = d_unit.p;
    a.ns = ns;
    a.g = g7;
    auto with_obs_normals = [](int k) { return k == EL_ADJ || k == EL_HYP; };
    // P2P: the source points with densities w x
    a.kid = kid;
    a.kp = make_kparams(kid, mu, nu);
    a.want_n = with_obs_normals(kid);
    a.s_xyz = dsrc->xyz.p;
    a.s_nrm = dsrc->nrm64.p;
    a.s_v = xt;
    a.s_n = NS;
    grad_pass(p2p, false, a, s, &launches);
    // M2P and L2P: equivalent surfaces, the kernel that reaches the targets
    a.kid = f.kt_kid;
    a.kp = make_kparams(f.kt_kid, mu, nu);
    a.want_n = with_obs_normals(f.kt_kid);
    if (!L.m2p.empty()) {
        a.q32 = nullptr;
        a.q64 = f.f64 ? cu64.p : qu64.p;
        a.s_center = dsrc->center.p;
        a.s_rad = dsrc->rad.p;
        a.s_rref = f.r_ue;
        grad_pass(m2p, true, a, s, &launches);
    }
    a.q32 = nullptr;
    a.q64 = qdn;
    a.s_center = dobs.center.p;
    a.s_rad = dobs.rad.p;
    a.s_rref = f.r_de;
    grad_pass(l2p, true, a, s, &launches);
    grad_scatter_kernel<<<blocks_for(NO), 256, 0, s>>>(g7, dobs.perm.p, nullptr, NO, gu, gu + 3 * NO,
                                                       nullptr);
    TBEM_CK(cudaGetLastError());
    if (g_x) TBEM_CK(cudaMemcpyAsync(g_x, gu, sizeof(double) * 3 * NO, cudaMemcpyDefault, s));
    if (g_n) TBEM_CK(cudaMemcpyAsync(g_n, gu + 3 * NO, sizeof(double) * 3 * NO, cudaMemcpyDefault, s));
    check_tc_flags(true, s);
}

}  // namespace tbem

extern "C" int tbem_direct_gradients(int kernel, const double* kernel_params,
                                     const double* obs_locs, const double* obs_normals, long n_obs,
                                     const double* src_locs, const double* src_normals,
                                     const double* src_weights, long n_src, const double* x,
                                     const double* r, double* g_obs_locs, double* g_obs_normals,
                                     double* g_src_locs, double* g_src_normals,
                                     double* g_src_weights, double* g_x, void* stream)
{
    using namespace tbem;
    try {
        if (kernel < 0 || kernel > 6 || n_obs < 0 || n_src < 0) throw Error(TBEM_ERR_ARG, "bad argument");
        const int R = kernel_dim(kernel);
        const double mu = (kernel_params && R == 3) ? kernel_params[0] : 1.0;
        const double nu = (kernel_params && R == 3) ? kernel_params[1] : 0.25;
        const KParams kp = make_kparams(kernel, mu, nu);
        cudaStream_t s = (cudaStream_t)stream;
        In ol, on, sl, sn, sw, xs, rs;
        ol.stage(obs_locs, 3 * n_obs, s);
        on.stage(obs_normals, 3 * n_obs, s);
        sl.stage(src_locs, 3 * n_src, s);
        sn.stage(src_normals, 3 * n_src, s);
        sw.stage(src_weights, n_src, s);
        xs.stage(x, (size_t)R * n_src, s);
        rs.stage(r, (size_t)R * n_obs, s);
        Out go, gno, gs, gns, gw, gx;
        go.stage(g_obs_locs, 3 * n_obs);
        gno.stage(g_obs_normals, 3 * n_obs);
        gs.stage(g_src_locs, 3 * n_src);
        gns.stage(g_src_normals, 3 * n_src);
        gw.stage(g_src_weights, n_src);
        gx.stage(g_x, (size_t)R * n_src);
        if (n_src > 0 && (gs.p || gns.p || gw.p || gx.p)) {
            if (n_obs == 0) {
                for (Out* o : {&gs, &gns, &gw, &gx})
                    if (o->p) TBEM_CK(cudaMemsetAsync(o->p, 0, o->n * sizeof(double), s));
            } else {
                grad_src_kernel<<<(unsigned)((n_src + 127) / 128), 128, 0, s>>>(
                    kernel, kp, ol.p, on.p, n_obs, sl.p, sn.p, sw.p, n_src, xs.p, rs.p, gs.p, gns.p,
                    gw.p, gx.p);
                TBEM_CK(cudaGetLastError());
            }
        }
        if (n_obs > 0 && (go.p || gno.p)) {
            if (n_src == 0) {
                for (Out* o : {&go, &gno})
                    if (o->p) TBEM_CK(cudaMemsetAsync(o->p, 0, o->n * sizeof(double), s));
            } else {
                grad_obs_kernel<<<(unsigned)((n_obs + 127) / 128), 128, 0, s>>>(
                    kernel, kp, ol.p, on.p, n_obs, sl.p, sn.p, sw.p, n_src, xs.p, rs.p, go.p, gno.p);
                TBEM_CK(cudaGetLastError());
            }
        }
        for (Out* o : {&go, &gno, &gs, &gns, &gw, &gx}) o->finish(s);
        TBEM_CK(cudaStreamSynchronize(s));
        return TBEM_OK;
    } catch (...) {
        return tbem::api_status();
    }
}
