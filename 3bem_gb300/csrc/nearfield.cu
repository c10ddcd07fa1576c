// Nearfield / farfield-correction matrix construction on the GPU.
//
// The reference builds these sparse matrices term by term on the host
// (make_nearfield_operator / make_farfield_correction_operator,
// cpp/nearfield_operator.h:48-117): for every Galerkin observation point and
// every source facet near it, IntegrationStrategy::compute_term
// (cpp/integral_term.cpp:33-92) integrates the kernel times the facet's
// linear basis by one of three rules -- a fixed Gauss rule far away, a
// sinh-transformed Gauss rule nearby (SinhIntegrator,
// cpp/integral_term.cpp:155-203, with the transforms of cpp/gauss_quad.cpp:
// 54-90 and cpp/sinh_quad.cpp), and, for observation points on the surface,
// Richardson extrapolation (cpp/richardson.h) of nearby integrals taken at
// points stepped back along the limit direction.
//
// Here the host finds the terms (nearfield_host.cpp) and classifies each one
// exactly as compute_term does (closest point, far / near / singular); a
// singular term becomes one near evaluation per Richardson step at the
// stepped-back point, computed on the host like the reference's
// get_step_loc.  The GPU integrates every evaluation: one warp per
// evaluation, the lanes striding over its quadrature points (every node
// generated on the fly from a table of Gauss rules) and meeting in a
// butterfly reduction.  The host extrapolates the singular terms
// (richardson_limit), lays the values out as the reference's COO entries and
// compresses them to CSR (csr_from_coo's stable row order).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "handle.h"
#include "nearfield.h"

namespace tbem {
namespace {

constexpr int NF_GMAX = 512;  // largest Gauss rule the device table holds
constexpr int NF_WARPS = 4;   // terms per CTA

struct NfArgs {
    int kid;
    KParams kp;
    int sinh_order;
    const double* gx;  // Gauss rule n (n = 1..NF_GMAX) at offset n (n - 1) / 2
    const double* gw;
    const double* fx;  // source farfield rule: [n_far][2] reference points
    const double* fw;
    int n_far;
    const double* loc;  // evaluation points [n_items][3]
    const double* nrm;  // observation normals [n_obs][3]
    const double* fac;  // source facets [n][3 corners][3]
    const double* ls;   // length scale
    const double* jac;  // jacobian
    const double* fn;   // facet normal [n][3]
    const int* i_obs;   // per evaluation: observation point (for its normal),
    const int* i_fac;   // source facet,
    const int* i_near;  // 1: sinh rule at the point, 0: the farfield rule, 2: skipped here
    long n_items;
    double* out;  // [n_items][dim][R][C]
    int* err;     // bit 1: a point on a facet; bit 2: rule too large
};

__device__ __forceinline__ double gnode(const NfArgs& a, int n, int i) { return a.gx[n * (n - 1) / 2 + i]; }
__device__ __forceinline__ double gweight(const NfArgs& a, int n, int i) { return a.gw[n * (n - 1) / 2 + i]; }

struct DClosest {
    double ref0, ref1, dist;
};

// nf::closest_point on the device, formula for formula.
template <int DIM>
__device__ DClosest d_closest(const double* p, const double* c)
{
    DClosest r{0.0, 0.0, 0.0};
    if (DIM == 2) {
        const double dx = c[3] - c[0], dy = c[4] - c[1];
        const double L2 = dx * dx + dy * dy;
        double t = 0.0;
        if (L2 > 0.0) {
            t = ((p[0] - c[0]) * dx + (p[1] - c[1]) * dy) / L2;
            t = fmin(1.0, fmax(0.0, t));
        }
        double qx, qy;
        if (t == 1.0) { qx = c[3]; qy = c[4]; }
        else if (t == 0.0) { qx = c[0]; qy = c[1]; }
        else { qx = c[0] + dx * t; qy = c[1] + dy * t; }
        r.ref0 = 2 * t - 1;
        r.dist = sqrt((p[0] - qx) * (p[0] - qx) + (p[1] - qy) * (p[1] - qy));
        return r;
    }
    double ab[3], ac[3], ap[3], bp[3], cp[3];
    for (int d = 0; d < 3; d++) {
        ab[d] = c[3 + d] - c[d];
        ac[d] = c[6 + d] - c[d];
        ap[d] = p[d] - c[d];
        bp[d] = p[d] - c[3 + d];
        cp[d] = p[d] - c[6 + d];
    }
    auto dot = [](const double* u, const double* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
    const double d1 = dot(ab, ap), d2 = dot(ac, ap), d3 = dot(ab, bp), d4 = dot(ac, bp);
    const double d5 = dot(ab, cp), d6 = dot(ac, cp);
    const double vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
    double v = 0.0, w = 0.0, q[3];
    if (d1 <= 0.0 && d2 <= 0.0) {
        for (int d = 0; d < 3; d++) q[d] = c[d];
    } else if (d3 >= 0.0 && d4 <= d3) {
        v = 1.0;
        for (int d = 0; d < 3; d++) q[d] = c[3 + d];
    } else if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        v = d1 / (d1 - d3);
        for (int d = 0; d < 3; d++) q[d] = c[d] + ab[d] * v;
    } else if (d6 >= 0.0 && d5 <= d6) {
        w = 1.0;
        for (int d = 0; d < 3; d++) q[d] = c[6 + d];
    } else if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        w = d2 / (d2 - d6);
        for (int d = 0; d < 3; d++) q[d] = c[d] + ac[d] * w;
    } else if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
        w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        v = 1.0 - w;
        for (int d = 0; d < 3; d++) q[d] = c[3 + d] + (c[6 + d] - c[3 + d]) * w;
    } else {
        const double inv = 1.0 / (va + vb + vc);
        v = vb * inv;
        w = vc * inv;
        for (int d = 0; d < 3; d++) q[d] = c[d] + ab[d] * v + ac[d] * w;
    }
    r.ref0 = v;
    r.ref1 = w;
    r.dist = sqrt((p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) +
                  (p[2] - q[2]) * (p[2] - q[2]));
    return r;
}

// One source quadrature point's influence (IntegralTerm::eval_point_influence,
// cpp/integral_term.cpp:11-20): basis (x) K(obs, y(x_hat)) * jacobian * w.
template <int DIM, int R>
__device__ __forceinline__ void influence(const NfArgs& a, int f, const double* p, const double* pn,
                                          double xh0, double xh1, double w, double* acc)
{
    const double* c = a.fac + 9 * f;
    double y[3], bas[3];
    // ref_to_real (cpp/numerics.h:81-100): left to right, every product
    // rounded (no contraction), the positions the farfield's source points
    // have too -- near a facet the kernel turns a one-ulp move of the point
    // into ~1e-12 of a ~1e5 entry, which the farfield and this correction only
    // cancel when both see the same point
    if (DIM == 2) {
        bas[0] = __dsub_rn(0.5, __dmul_rn(0.5, xh0));
        bas[1] = __dadd_rn(0.5, __dmul_rn(0.5, xh0));
        y[0] = __dadd_rn(__dmul_rn(bas[0], c[0]), __dmul_rn(bas[1], c[3]));
        y[1] = __dadd_rn(__dmul_rn(bas[0], c[1]), __dmul_rn(bas[1], c[4]));
        y[2] = 0.0;
    } else {
        bas[0] = __dsub_rn(__dsub_rn(1.0, xh0), xh1);
        bas[1] = xh0;
        bas[2] = xh1;
        for (int d = 0; d < 3; d++)
            y[d] = __dadd_rn(__dadd_rn(__dmul_rn(bas[0], c[d]), __dmul_rn(bas[1], c[3 + d])),
                             __dmul_rn(bas[2], c[6 + d]));
    }
    double K[9];
    const double* n = a.fn + 3 * f;
    kernel_tensor_any<double>(a.kid, y[0] - p[0], y[1] - p[1], y[2] - p[2], pn[0], pn[1], pn[2], n[0],
                              n[1], n[2], a.kp, K);
    const double J = a.jac[f];
#pragma unroll
    for (int b = 0; b < DIM; b++)
#pragma unroll
        for (int k = 0; k < R * R; k++) acc[b * R * R + k] += bas[b] * (K[k] * J) * w;
}

// The sinh-transformed rule around the closest point (choose_sinh_quad +
// sinh_transform / sinh_sigmoidal_transform), this lane's share.  Returns
// false (and flags) when the point lies on the facet or the rule is too big.
template <int DIM, int R>
__device__ bool sinh_near(const NfArgs& a, int f, const double* p, const double* pn, double* acc)
{
    const int lane = threadIdx.x & 31;
    const DClosest cp = d_closest<DIM>(p, a.fac + 9 * f);
    const double l = cp.dist, S = a.ls[f];
    if (!(l > 0.0)) {
        if (lane == 0) atomicOr(a.err, 1);
        return false;
    }
    const double scaled = l / S;
    int n = (int)(a.sinh_order + (a.sinh_order * (-log(scaled))));
    n = max(n, a.sinh_order);
    if ((DIM == 3 ? 2 * n : n) > NF_GMAX) {
        if (lane == 0) atomicOr(a.err, 2);
        return false;
    }
    const double sa = DIM == 3 ? -1.0 : cp.ref0, b = scaled;
    const double mu0 = 0.5 * (asinh((1.0 + sa) / b) + asinh((1.0 - sa) / b));
    const double eta0 = 0.5 * (asinh((1.0 + sa) / b) - asinh((1.0 - sa) / b));
    if (DIM == 2) {
        for (int q = lane; q < n; q += 32) {
            const double s = gnode(a, n, q);
            const double x = sa + b * sinh(mu0 * s - eta0);
            const double jw = b * mu0 * cosh(mu0 * s - eta0);
            influence<DIM, R>(a, f, p, pn, x, 0.0, gweight(a, n, q) * jw, acc);
        }
        return true;
    }
    // three sub-triangles around the singular point (x0, y0): {sp, p0, p2},
    // {sp, p2, p1}, {sp, p0, p1} with p0 = (0,0), p1 = (1,0), p2 = (0,1)
    const double x0 = cp.ref0, y0 = cp.ref1;
    const double tx[3][3] = {{x0, 0.0, 0.0}, {x0, 0.0, 1.0}, {x0, 0.0, 1.0}};
    const double ty[3][3] = {{y0, 0.0, 1.0}, {y0, 1.0, 0.0}, {y0, 0.0, 0.0}};
    double tj[3];
#pragma unroll
    for (int t = 0; t < 3; t++) {  // 2 * tri_area = |cross(c2 - c0, c2 - c1)_z|
        const double ux = tx[t][2] - tx[t][0], uy = ty[t][2] - ty[t][0];
        const double vx = tx[t][2] - tx[t][1], vy = ty[t][2] - ty[t][1];
        tj[t] = 2.0 * (0.5 * fabs(ux * vy - uy * vx));
    }
    const int nt = 2 * n, per = nt * n;
    const double hp = M_PI / 2.0, s45 = sin(M_PI / 4.0);
    for (int q = lane; q < 3 * per; q += 32) {
        const int t = q / per, rem = q - t * per, i = rem / n, j = rem - i * n;
        const double u = gnode(a, nt, i);
        const double sigma = (u + 1.0) / 2.0;
        const double s2 = sigma * sigma, c2 = (1 - sigma) * (1 - sigma);
        const double theta = s2 / (s2 + c2) * hp;
        const double theta_j = hp * sigma * (1 - sigma) / ((s2 + c2) * (s2 + c2));
        const double Rt = s45 / sin(theta + M_PI / 4.0);
        const double s = gnode(a, n, j);
        const double xs = sa + b * sinh(mu0 * s - eta0);
        const double ws = gweight(a, n, j) * (b * mu0 * cosh(mu0 * s - eta0));
        const double r = Rt * (xs + 1.0) / 2.0;
        const double rj = r * (Rt / 2.0);
        const double w = theta_j * rj * ws * gweight(a, nt, i);
        const double ux = r * cos(theta), uy = r * sin(theta);
        const double b0 = 1 - ux - uy;
        const double px = b0 * tx[t][0] + ux * tx[t][1] + uy * tx[t][2];
        const double py = b0 * ty[t][0] + ux * ty[t][1] + uy * ty[t][2];
        influence<DIM, R>(a, f, p, pn, px, py, w * tj[t], acc);
    }
    return true;
}

template <int E>
__device__ __forceinline__ void warp_sum(double* acc)
{
#pragma unroll
    for (int e = 0; e < E; e++)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc[e] += __shfl_xor_sync(0xffffffffu, acc[e], off);
}

template <int DIM, int R>
__global__ void __launch_bounds__(32 * NF_WARPS) nearfield_kernel(const NfArgs a)
{
    constexpr int E = DIM * R * R;
    const long i = (long)blockIdx.x * NF_WARPS + threadIdx.x / 32;
    if (i >= a.n_items) return;  // whole warps leave together
    if (a.i_near[i] == 2) return;  // integrated by the adaptive rule instead
    const int lane = threadIdx.x & 31;
    const int f = a.i_fac[i];
    const double* p = a.loc + 3 * i;
    const double* pn = a.nrm + 3 * a.i_obs[i];
    double acc[E];
#pragma unroll
    for (int e = 0; e < E; e++) acc[e] = 0.0;
    if (a.i_near[i]) {
        sinh_near<DIM, R>(a, f, p, pn, acc);
    } else {
        for (int q = lane; q < a.n_far; q += 32)
            influence<DIM, R>(a, f, p, pn, a.fx[2 * q], a.fx[2 * q + 1], a.fw[q], acc);
    }
    warp_sum<E>(acc);
    double result = 0.0;  // entry `lane` of the evaluation (lanes < E)
#pragma unroll
    for (int e = 0; e < E; e++)
        if (e == lane) result = acc[e];
    if (lane < E) a.out[i * E + lane] = result;
}

// The adaptive rule's points: one thread per point, the term's basis x
// kernel x jacobian at the reference point (eval_point_influence,
// cpp/integral_term.cpp:11-20).
template <int DIM, int R>
__global__ void point_influence_kernel(const NfArgs a, const int* p_item, const double* p_x0,
                                       const double* p_x1, long n, double* out)
{
    constexpr int E = DIM * R * R;
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = p_item[k];
    double acc[E];
#pragma unroll
    for (int e = 0; e < E; e++) acc[e] = 0.0;
    influence<DIM, R>(a, a.i_fac[i], a.loc + 3 * i, a.nrm + 3 * a.i_obs[i], p_x0[k], p_x1[k], 1.0, acc);
#pragma unroll
    for (int e = 0; e < E; e++) out[k * E + e] = acc[e];
}

template <int DIM, int R>
void launch_points(const NfArgs& a, const int* item, const double* x0, const double* x1, long n,
                   double* out)
{
    if (n <= 0) return;
    point_influence_kernel<DIM, R><<<(unsigned)((n + 127) / 128), 128>>>(a, item, x0, x1, n, out);
    TBEM_CK(cudaGetLastError());
}

// Gauss rules 1..NF_GMAX, computed once per process.
const std::vector<double>& gauss_table(int which)
{
    static std::vector<double> x, w;
    static std::once_flag once;
    std::call_once(once, [] {
        x.reserve((size_t)NF_GMAX * (NF_GMAX + 1) / 2);
        w.reserve(x.capacity());
        std::vector<double> gx, gw;
        for (int n = 1; n <= NF_GMAX; n++) {
            nf::gauss_rule(n, gx, gw);
            x.insert(x.end(), gx.begin(), gx.end());
            w.insert(w.end(), gw.begin(), gw.end());
        }
    });
    return which == 0 ? x : w;
}

std::vector<nf::Facet> read_facets(const double* verts, long n_verts, const long* idx, long n, int dim)
{
    if (n > 0 && (!idx || !verts)) throw Error(TBEM_ERR_ARG, "null vertex or facet array");
    // facet and point numbers travel to the device as int
    if (n > (long)INT32_MAX) throw Error(TBEM_ERR_ARG, "too many facets");
    std::vector<nf::Facet> out((size_t)n);
    for (long i = 0; i < n; i++) {
        nf::Facet f{};
        for (int v = 0; v < dim; v++) {
            const long k = idx[dim * i + v];
            if (k < 0 || k >= n_verts) throw Error(TBEM_ERR_ARG, "facet vertex index out of range");
            for (int d = 0; d < dim; d++) f.c[v][d] = verts[dim * k + d];
        }
        out[i] = f;
    }
    return out;
}

template <int DIM, int R>
void launch(const NfArgs& a)
{
    const long blocks = (a.n_items + NF_WARPS - 1) / NF_WARPS;
    nearfield_kernel<DIM, R><<<(unsigned)blocks, 32 * NF_WARPS>>>(a);
    TBEM_CK(cudaGetLastError());
}

// The nearfield (which 0) or farfield-correction (which 1) CSR of the
// observation points pts against the source facets (the body of
// nearfield_inner_integral, cpp/nearfield_operator.h:48-95).
int build_nearfield_csr(int kernel, int dim, int R, double mu, double nu, const nf::ObsPoints& pts,
                        const std::vector<nf::Facet>& src, const nf::FacetSet& src_set,
                        const TbemIntegrator* mthd, int which, TbemCsr** out)
{
    const long n_pts = (long)pts.loc.size();
    if (n_pts > (long)INT32_MAX) throw Error(TBEM_ERR_ARG, "too many observation points");

    // every (point, nearfield facet) term in the reference's order, classified
    // as IntegrationStrategy::compute_term does (far / near / singular), with
    // its evaluations: one for a far or near term, n_steps at the stepped-back
    // points for a singular one; the correction matrix (which 1) is
    // -compute_farfield of every term (host, all cores)
    const int E = dim * R * R;
    const int n_steps = (int)mthd->n_singular_steps;
    nf::TermPlan tp = nf::plan_terms(pts, src, src_set, mthd->far_threshold, n_steps, dim, which == 1);
    if (tp.on_facet && mthd->strategy == TBEM_QUAD_SINH)
        throw Error(TBEM_ERR_ARG, "an observation point lies on a source facet without a "
                                  "limit direction (the reference's sinh rule asserts here)");
    const std::vector<int>&i_obs = tp.i_obs, &i_fac = tp.i_fac;
    std::vector<int>& i_near = tp.i_near;
    const std::vector<double>& iloc = tp.iloc;
    const long n_items = (long)i_obs.size();
    // the adaptive evaluations name their item as int on the device
    if (n_items > (long)INT32_MAX) throw Error(TBEM_ERR_ARG, "too many nearfield terms");
    const bool adaptive = mthd->strategy == TBEM_QUAD_ADAPTIVE;
    std::vector<long> adaptive_items;  // near evaluations done by the adaptive rule
    if (adaptive)
        for (long i = 0; i < n_items; i++)
            if (i_near[i] == 1) {
                i_near[i] = 2;
                adaptive_items.push_back(i);
            }
    std::vector<double> ivals((size_t)n_items * E);
    if (n_items > 0) {
        std::vector<double> nrm, fac, ls, jac, fn;
        for (long i = 0; i < n_pts; i++)
            for (int d = 0; d < 3; d++) nrm.push_back(pts.normal[i][d]);
        for (size_t f = 0; f < src.size(); f++) {
            for (int v = 0; v < 3; v++)
                for (int d = 0; d < 3; d++) fac.push_back(src[f].c[v][d]);
            const nf::FacetInfo& fi = src_set.info(f);
            ls.push_back(fi.length_scale);
            jac.push_back(fi.jacobian);
            for (int d = 0; d < 3; d++) fn.push_back(fi.normal[d]);
        }
        std::vector<double> fx, fw;
        nf::gauss_facet(dim, (int)mthd->src_far_order, fx, fw);
        DBuf<double> d_gx, d_gw, d_fx, d_fw, d_loc, d_nrm, d_fac, d_ls, d_jac, d_fn, d_out;
        DBuf<int> d_io, d_if, d_in, d_err;
        d_gx.upload(gauss_table(0));
        d_gw.upload(gauss_table(1));
        d_fx.upload(fx);
        d_fw.upload(fw);
        d_loc.upload(iloc);
        d_nrm.upload(nrm);
        d_fac.upload(fac);
        d_ls.upload(ls);
        d_jac.upload(jac);
        d_fn.upload(fn);
        d_io.upload(i_obs);
        d_if.upload(i_fac);
        d_in.upload(i_near);
        d_err.upload(std::vector<int>(1, 0));
        d_out.alloc(ivals.size());
        NfArgs a{};
        a.kid = kernel;
        a.kp = make_kparams(kernel, mu, nu);
        a.sinh_order = (int)mthd->sinh_order;
        a.gx = d_gx.p;
        a.gw = d_gw.p;
        a.fx = d_fx.p;
        a.fw = d_fw.p;
        a.n_far = (int)fw.size();
        a.loc = d_loc.p;
        a.nrm = d_nrm.p;
        a.fac = d_fac.p;
        a.ls = d_ls.p;
        a.jac = d_jac.p;
        a.fn = d_fn.p;
        a.i_obs = d_io.p;
        a.i_fac = d_if.p;
        a.i_near = d_in.p;
        a.n_items = n_items;
        a.out = d_out.p;
        a.err = d_err.p;
        if (dim == 2 && R == 1) launch<2, 1>(a);
        else if (dim == 2) launch<2, 2>(a);
        else if (R == 1) launch<3, 1>(a);
        else launch<3, 3>(a);
        TBEM_CK(cudaDeviceSynchronize());
        int err = 0;
        TBEM_CK(cudaMemcpy(&err, d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (err & 1)
            throw Error(TBEM_ERR_ARG, "a stepped-back Richardson point lies on a source facet");
        if (err & 2)
            throw Error(TBEM_ERR_ARG, "a sinh rule needs more than 512 Gauss points "
                                      "(observation point too close to a facet)");
        TBEM_CK(cudaMemcpy(ivals.data(), d_out.p, ivals.size() * sizeof(double),
                           cudaMemcpyDeviceToHost));
        if (!adaptive_items.empty()) {
            // the adaptive Gauss-Lobatto rule: subdivision on the host,
            // every level's points on the GPU
            // buffers kept across the levels (each level's batch has its own size)
            DBuf<int> d_pi;
            DBuf<double> d_x0, d_x1, d_pv;
            std::vector<int> it;
            nf::InfluenceEval eval = [&](const std::vector<long>& item, const std::vector<double>& x0,
                                         const std::vector<double>& x1, std::vector<double>& out) {
                const long n = (long)item.size();
                out.resize((size_t)n * E);  // every value is copied back below
                if (n == 0) return;
                it.resize(n);
                nf::parallel_for(n, [&](long k) { it[k] = (int)adaptive_items[item[k]]; }, 1 << 16);
                d_pi.upload_grow(it);
                d_x0.upload_grow(x0);
                d_x1.upload_grow(x1);
                d_pv.ensure((size_t)n * E);
                if (dim == 2 && R == 1) launch_points<2, 1>(a, d_pi.p, d_x0.p, d_x1.p, n, d_pv.p);
                else if (dim == 2) launch_points<2, 2>(a, d_pi.p, d_x0.p, d_x1.p, n, d_pv.p);
                else if (R == 1) launch_points<3, 1>(a, d_pi.p, d_x0.p, d_x1.p, n, d_pv.p);
                else launch_points<3, 3>(a, d_pi.p, d_x0.p, d_x1.p, n, d_pv.p);
                TBEM_CK(cudaMemcpy(out.data(), d_pv.p, out.size() * sizeof(double),
                                   cudaMemcpyDeviceToHost));
            };
            const std::vector<double> v = nf::adaptive_facet_integrals(
                dim, E, (long)adaptive_items.size(), mthd->near_tol, eval);
            for (size_t k = 0; k < adaptive_items.size(); k++)
                for (int e = 0; e < E; e++)
                    ivals[(size_t)adaptive_items[k] * E + e] = v[k * E + e];
        }
    }
    // Richardson limits / negation and the reference's CSR layout (host, all cores)
    std::vector<double> v;
    std::vector<long> cols, row_ptr;
    nf::assemble_csr(tp, ivals, n_pts, (long)src.size(), dim, R, n_steps, which == 1, v, cols, row_ptr);
    return tbem_csr_create(R * n_pts, R * (long)src.size() * dim, v.data(), cols.data(), row_ptr.data(),
                           out);
}

void validate(int kernel, int which, const TbemIntegrator* mthd)
{
    if (!kernel_valid(kernel)) throw Error(TBEM_ERR_ARG, "unknown kernel id");
    if (which != 0 && which != 1) throw Error(TBEM_ERR_ARG, "which must be 0 or 1");
    if (mthd->strategy != TBEM_QUAD_SINH && mthd->strategy != TBEM_QUAD_ADAPTIVE)
        throw Error(TBEM_ERR_ARG, "bad integrator parameters: unknown strategy");
    if ((mthd->strategy == TBEM_QUAD_SINH && mthd->sinh_order <= 0) ||
        (mthd->strategy == TBEM_QUAD_ADAPTIVE && !(mthd->near_tol > 0)) ||
        mthd->obs_near_order <= 0 || mthd->obs_far_order <= 0 || mthd->src_far_order <= 0 ||
        mthd->n_singular_steps < 2 || mthd->n_singular_steps > 32 || !(mthd->far_threshold > 0))
        throw Error(TBEM_ERR_ARG, "bad integrator parameters");
}

}  // namespace
}  // namespace tbem

extern "C" {

long tbem_gauss_facet(int dim, long n, double* x, double* w)
{
    try {
        if ((dim != 2 && dim != 3) || n <= 0 || n > 4096)
            throw tbem::Error(TBEM_ERR_ARG, "dim must be 2 or 3 and n in [1, 4096]");
        std::vector<double> qx, qw;
        tbem::nf::gauss_facet(dim, (int)n, qx, qw);
        if (x)
            for (size_t i = 0; i < qw.size(); i++) {
                x[(dim - 1) * i] = qx[2 * i];
                if (dim == 3) x[2 * i + 1] = qx[2 * i + 1];
            }
        if (w) std::copy(qw.begin(), qw.end(), w);
        return (long)qw.size();
    } catch (...) {
        return tbem::api_status();
    }
}

long tbem_galerkin_obs_points(int dim, const double* vertices, long n_vertices,
                              const long* obs_facets, long n_obs_facets, const long* all_facets,
                              long n_all_facets, long order, double* locs, double* normals,
                              double* dirs)
{
    using namespace tbem;
    try {
        if ((dim != 2 && dim != 3) || order <= 0 || n_vertices < 0 || n_obs_facets < 0 || n_all_facets < 0)
            throw Error(TBEM_ERR_ARG, "bad argument");
        const auto obs = read_facets(vertices, n_vertices, obs_facets, n_obs_facets, dim);
        const auto all = read_facets(vertices, n_vertices, all_facets, n_all_facets, dim);
        nf::FacetSet all_set(all, dim);
        const nf::ObsPoints pts = nf::galerkin_obs_points(obs, all_set, (int)order, dim);
        for (size_t i = 0; i < pts.loc.size(); i++)
            for (int d = 0; d < dim; d++) {
                if (locs) locs[dim * i + d] = pts.loc[i][d];
                if (normals) normals[dim * i + d] = pts.normal[i][d];
                if (dirs) dirs[dim * i + d] = pts.dir[i][d];
            }
        return (long)pts.loc.size();
    } catch (...) {
        return tbem::api_status();
    }
}

int tbem_nearfield_create(int kernel, const double* kernel_params, const double* vertices,
                          long n_vertices, const long* obs_facets, long n_obs_facets,
                          const long* src_facets, long n_src_facets, const long* all_facets,
                          long n_all_facets, const TbemIntegrator* mthd, int which,
                          TbemCsr** out)
{
    using namespace tbem;
    if (!out || !mthd) return TBEM_ERR_ARG;
    *out = nullptr;
    try {
        validate(kernel, which, mthd);
        if (n_vertices < 0 || n_obs_facets < 0 || n_src_facets < 0 || n_all_facets < 0)
            throw Error(TBEM_ERR_ARG, "negative count");
        const int dim = kernel_space_dim(kernel), R = kernel_dim(kernel);
        const double mu = (kernel_params && R > 1) ? kernel_params[0] : 1.0;
        const double nu = (kernel_params && R > 1) ? kernel_params[1] : 0.25;
        const auto obs = read_facets(vertices, n_vertices, obs_facets, n_obs_facets, dim);
        const auto src = read_facets(vertices, n_vertices, src_facets, n_src_facets, dim);
        const auto all = read_facets(vertices, n_vertices, all_facets, n_all_facets, dim);
        nf::FacetSet all_set(all, dim), src_set(src, dim);
        const int order = (int)(which == 0 ? mthd->obs_near_order : mthd->obs_far_order);
        const nf::ObsPoints pts = nf::galerkin_obs_points(obs, all_set, order, dim);
        return build_nearfield_csr(kernel, dim, R, mu, nu, pts, src, src_set, mthd, which, out);
    } catch (...) {
        return tbem::api_status();
    }
}

long tbem_interior_obs_points(int dim, const double* locs, long n, const double* vertices,
                              long n_vertices, const long* all_facets, long n_all_facets,
                              double* dirs)
{
    using namespace tbem;
    try {
        if ((dim != 2 && dim != 3) || n < 0 || n_vertices < 0 || n_all_facets < 0 || (n > 0 && !locs))
            throw Error(TBEM_ERR_ARG, "bad argument");
        const auto all = read_facets(vertices, n_vertices, all_facets, n_all_facets, dim);
        nf::FacetSet all_set(all, dim);
        nf::parallel_for(n, [&](long i) {
            nf::V3 p{{0, 0, 0}};
            for (int d = 0; d < dim; d++) p[d] = locs[dim * i + d];
            const nf::V3 r = nf::limit_direction(p, all_set, dim);
            if (dirs)
                for (int d = 0; d < dim; d++) dirs[dim * i + d] = r[d];
        });
        return n;
    } catch (...) {
        return tbem::api_status();
    }
}

int tbem_nearfield_points_create(int kernel, const double* kernel_params, const double* obs_locs,
                                 const double* obs_normals, long n_obs, const double* vertices,
                                 long n_vertices, const long* src_facets, long n_src_facets,
                                 const long* all_facets, long n_all_facets,
                                 const TbemIntegrator* mthd, int which, TbemCsr** out)
{
    using namespace tbem;
    if (!out || !mthd) return TBEM_ERR_ARG;
    *out = nullptr;
    try {
        validate(kernel, which, mthd);
        if (n_obs < 0 || n_vertices < 0 || n_src_facets < 0 || n_all_facets < 0)
            throw Error(TBEM_ERR_ARG, "negative count");
        if (n_obs > 0 && (!obs_locs || !obs_normals)) throw Error(TBEM_ERR_ARG, "null point array");
        const int dim = kernel_space_dim(kernel), R = kernel_dim(kernel);
        const double mu = (kernel_params && R > 1) ? kernel_params[0] : 1.0;
        const double nu = (kernel_params && R > 1) ? kernel_params[1] : 0.25;
        const auto src = read_facets(vertices, n_vertices, src_facets, n_src_facets, dim);
        const auto all = read_facets(vertices, n_vertices, all_facets, n_all_facets, dim);
        nf::FacetSet all_set(all, dim), src_set(src, dim);
        // interior_obs_pts (cpp/nearfield_operator.h:27-40): the given points and
        // normals with their limit directions against all_facets
        nf::ObsPoints pts;
        for (long i = 0; i < n_obs; i++) {
            nf::V3 p{{0, 0, 0}}, nn{{0, 0, 0}};
            for (int d = 0; d < dim; d++) {
                p[d] = obs_locs[dim * i + d];
                nn[d] = obs_normals[dim * i + d];
            }
            pts.loc.push_back(p);
            pts.normal.push_back(nn);
        }
        pts.dir.resize(n_obs);
        nf::parallel_for(n_obs, [&](long i) { pts.dir[i] = nf::limit_direction(pts.loc[i], all_set, dim); });
        return build_nearfield_csr(kernel, dim, R, mu, nu, pts, src, src_set, mthd, which, out);
    } catch (...) {
        return tbem::api_status();
    }
}

}  // extern "C"
