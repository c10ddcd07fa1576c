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

}  // namespace
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
