// Device-side BEM kernels, templated on the arithmetic type.
//
// Each kernel K(x, y; n_x, n_y) is an R x C tensor evaluated with
// delta = y - x and the reference's self-pair rule: zero when r^2 < 1e-12
// (cpp/kernel.h:19-33).  3D formulas: LaplaceSingle 1/(4 pi r)
// (cpp/laplace_kernels.h:25), LaplaceDouble n_y.delta/(4 pi r^3) (:41),
// ElasticDisplacement / Traction / AdjointTraction / Hypersingular
// (cpp/elastic_kernels.h:192-357), IdentityScalar (cpp/identity_kernels.h).
// 2D (ids 16-23, the kernels of FMMOperator<2,1,1> / <2,2,2>):
// LaplaceSingle log(r)/(2 pi), LaplaceDouble n_y.delta/(2 pi r^2),
// LaplaceHypersingular (cpp/laplace_kernels.h:66-110) and the 2x2 elastic
// kernels (cpp/elastic_kernels.h:21-189).  2D points live in the same
// [n][3] buffers with z = 0; the 2D formulas read x and y only.
//
// accumulate<KID, TRANS>() adds K v (or K^T v for the transposed apply) for
// one pair directly, without forming the tensor: the elastic kernels reduce
// to dot products with delta and the normals.  The kernel's leading constant
// (1/(4 pi), C1) is applied once per target by the caller (kernel_scale).
#pragma once
#include <cuda_runtime.h>

namespace tbem {

enum KernelId {
    LAP_S = 0, LAP_D = 1, EL_DISP = 2, EL_TRAC = 3, EL_ADJ = 4, IDENT = 5, EL_HYP = 6,
    LAP_S2 = 16, LAP_D2 = 17, LAP_H2 = 18, EL_DISP2 = 19, EL_TRAC2 = 20, EL_ADJ2 = 21,
    EL_HYP2 = 22, IDENT2 = 23
};

// Kernels whose value holds a normal component n . d of the separation d.
// For a nearly tangent pair on a curved surface n . d is O(kappa h^2) while
// the positions are O(cell width) from the FP32 origin, so FP32 separations
// cancel badly there; the FP32 point-to-point passes of these kernels carry
// the low parts of the positions as well (separation error O(eps |d|)).
__host__ __device__ constexpr bool normal_dot_kernel(int kid)
{
    return kid == LAP_D || kid == EL_TRAC || kid == EL_ADJ || kid == EL_HYP || kid == LAP_D2 ||
           kid == LAP_H2 || kid == EL_TRAC2 || kid == EL_ADJ2 || kid == EL_HYP2;
}

// R (= C): the number of components of the kernel's tensor
__host__ __device__ constexpr int kernel_dim(int kid)
{
    return (kid == EL_DISP || kid == EL_TRAC || kid == EL_ADJ || kid == EL_HYP) ? 3
           : (kid >= EL_DISP2 && kid <= EL_HYP2)                                ? 2
                                                                                : 1;
}

// the dimension of the space the kernel lives in
__host__ __device__ constexpr int kernel_space_dim(int kid) { return kid >= LAP_S2 ? 2 : 3; }

__host__ __device__ constexpr bool kernel_valid(int kid)
{
    return (kid >= LAP_S && kid <= EL_HYP) || (kid >= LAP_S2 && kid <= IDENT2);
}

// Constants of a kernel instance (mu, nu enter through c1, c2).
struct KParams {
    double scale;  // leading constant applied once per target
    double c2;     // second elastic constant (3-4nu for disp, 1-2nu for traction)
};

inline KParams make_kparams(int kid, double mu, double nu)
{
    const double pi = 3.14159265358979323846;
    KParams p{1.0, 0.0};
    switch (kid) {
    case LAP_S: p.scale = 1.0 / (4.0 * pi); break;
    case LAP_D: p.scale = 1.0 / (4.0 * pi); break;
    case EL_DISP: p.scale = 1.0 / (16 * pi * mu * (1 - nu)); p.c2 = 3 - 4 * nu; break;
    case EL_TRAC:
    case EL_ADJ: p.scale = 1.0 / (8 * pi * (1 - nu)); p.c2 = 1 - 2 * nu; break;
    case EL_HYP: p.scale = mu / (4 * pi * (1 - nu)); p.c2 = 1 - 2 * nu; break;
    case LAP_S2:
    case LAP_D2:
    case LAP_H2: p.scale = 1.0 / (2.0 * pi); break;
    case EL_DISP2: p.scale = 1.0 / (8 * pi * mu * (1 - nu)); p.c2 = 3 - 4 * nu; break;
    case EL_TRAC2:
    case EL_ADJ2: p.scale = 1.0 / (4 * pi * (1 - nu)); p.c2 = 1 - 2 * nu; break;
    case EL_HYP2: p.scale = mu / (2 * pi * (1 - nu)); p.c2 = 1 - 2 * nu; break;
    default: p.scale = 1.0; break;
    }
    return p;
}

template <typename T>
__device__ __forceinline__ T dev_rsqrt(T x);
template <>
__device__ __forceinline__ double dev_rsqrt<double>(double x) { return rsqrt(x); }
template <>
__device__ __forceinline__ float dev_rsqrt<float>(float x) { return rsqrtf(x); }

template <typename T>
__device__ __forceinline__ T dev_log(T x);
template <>
__device__ __forceinline__ double dev_log<double>(double x) { return log(x); }
template <>
__device__ __forceinline__ float dev_log<float>(float x) { return logf(x); }

// 2D hypersingular tensor without the leading constant (cpp/elastic_kernels.h:
// 157-181): like the 3D one with the 2D exponents (r^-2; coefficients 2 and
// 4 where 3D has 3 and 5).  m: observation normal, n: source normal.
template <typename T>
__device__ __forceinline__ void hyp_tensor_2d(T dx, T dy, T ir, T mx, T my, T nx, T ny, T c2,
                                              T* H)
{
    const T nu = (T(1) - c2) * T(0.5);
    const T e[2] = {dx * ir, dy * ir};
    const T m[2] = {mx, my}, n[2] = {nx, ny};
    const T em = e[0] * mx + e[1] * my;
    const T en = e[0] * nx + e[1] * ny;
    const T nm = nx * mx + ny * my;
    const T C = ir * ir;
#pragma unroll
    for (int k = 0; k < 2; k++)
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const T dkj = k == j ? T(1) : T(0);
            const T t1 = T(2) * en * (c2 * m[k] * e[j] + nu * (m[j] * e[k] + dkj * em) -
                                      T(4) * e[k] * e[j] * em);
            const T t2 = c2 * (T(2) * n[j] * e[k] * em + dkj * nm + n[k] * m[j]);
            const T t3 = T(2) * nu * (n[k] * e[j] * em + nm * e[k] * e[j]);
            const T t4 = (T(4) * nu - T(1)) * n[j] * m[k];
            H[2 * k + j] = C * (t1 + t2 + t3 + t4);
        }
}

// Hypersingular tensor without the leading constant (cpp/elastic_kernels.h:
// 333-357): the traction (observation normal m) of the displacement field of
// a dislocation with normal n, r^-3 times a polynomial in e = d / r, m, n.
// nu comes from c2 = 1 - 2 nu.
template <typename T>
__device__ __forceinline__ void hyp_tensor(T dx, T dy, T dz, T r2, T ir, T mx, T my, T mz, T nx,
                                           T ny, T nz, T c2, T* H)
{
    const T nu = (T(1) - c2) * T(0.5);
    const T c3 = T(3) * nu, c4 = T(4) * nu - T(1);
    const T e[3] = {dx * ir, dy * ir, dz * ir};
    const T m[3] = {mx, my, mz}, n[3] = {nx, ny, nz};
    const T em = e[0] * mx + e[1] * my + e[2] * mz;
    const T en = e[0] * nx + e[1] * ny + e[2] * nz;
    const T nm = nx * mx + ny * my + nz * mz;
    const T C = ir / r2;
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const T dkj = k == j ? T(1) : T(0);
            const T t1 = T(3) * en * (c2 * m[k] * e[j] + nu * (m[j] * e[k] + dkj * em) -
                                      T(5) * e[k] * e[j] * em);
            const T t2 = c2 * (T(3) * n[j] * e[k] * em + dkj * nm + n[k] * m[j]);
            const T t3 = c3 * (n[k] * e[j] * em + nm * e[k] * e[j]);
            const T t4 = c4 * n[j] * m[k];
            H[3 * k + j] = C * (t1 + t2 + t3 + t4);
        }
}

// u += K(x,y) v  (TRANS: u += K(x,y)^T v), without the leading constant.
// d = y - x; no = n_x (observation normal), ns = n_y (source normal).
// Returns false (adds nothing) for the self pair.
template <int KID, bool TRANS, typename T>
__device__ __forceinline__ void accumulate(T dx, T dy, T dz, T nox, T noy, T noz, T nsx, T nsy,
                                           T nsz, T c2, const T* v, T* u)
{
    const T r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < T(1e-12)) return;
    const T ir = dev_rsqrt<T>(r2);
    if (KID == LAP_S) {
        u[0] += v[0] * ir;
    } else if (KID == LAP_D) {
        const T dn = nsx * dx + nsy * dy + nsz * dz;
        u[0] += v[0] * (dn * ir * ir * ir);
    } else if (KID == IDENT) {
        u[0] += v[0];
    } else if (KID == EL_DISP) {
        // K_kj = (1/r)(c2 delta_kj + d_k d_j / r^2): symmetric
        const T ir2 = ir * ir;
        const T t = (dx * v[0] + dy * v[1] + dz * v[2]) * ir2;
        u[0] += ir * (c2 * v[0] + dx * t);
        u[1] += ir * (c2 * v[1] + dy * t);
        u[2] += ir * (c2 * v[2] + dz * t);
    } else if (KID == EL_HYP) {
        T H[9];
        hyp_tensor<T>(dx, dy, dz, r2, ir, nox, noy, noz, nsx, nsy, nsz, c2, H);
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                if (!TRANS) u[k] += H[3 * k + j] * v[j];
                else u[j] += H[3 * k + j] * v[k];
            }
    } else if (KID == LAP_S2) {
        u[0] += v[0] * (T(0.5) * dev_log<T>(r2));
    } else if (KID == LAP_D2) {
        const T dn = nsx * dx + nsy * dy;
        u[0] += v[0] * (dn * ir * ir);
    } else if (KID == LAP_H2) {
        // (-(m.n) / r^2 + 2 (n.d)(m.d) / r^4): symmetric under d -> -d, m <-> n
        const T ir2 = ir * ir;
        const T dn = nsx * dx + nsy * dy, dm = nox * dx + noy * dy;
        const T nm = nsx * nox + nsy * noy;
        u[0] += v[0] * (ir2 * (T(2) * dn * dm * ir2 - nm));
    } else if (KID == IDENT2) {
        u[0] += v[0];
    } else if (KID == EL_DISP2) {
        // K_kj = -c2 delta_kj log r + d_k d_j / r^2: symmetric
        const T lr = T(0.5) * dev_log<T>(r2);
        const T t = (dx * v[0] + dy * v[1]) * (ir * ir);
        u[0] += -c2 * lr * v[0] + dx * t;
        u[1] += -c2 * lr * v[1] + dy * t;
    } else if (KID == EL_HYP2) {
        T H[4];
        hyp_tensor_2d<T>(dx, dy, ir, nox, noy, nsx, nsy, c2, H);
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
            for (int j = 0; j < 2; j++) {
                if (!TRANS) u[k] += H[2 * k + j] * v[j];
                else u[j] += H[2 * k + j] * v[k];
            }
    } else if (KID == EL_TRAC2 || KID == EL_ADJ2) {
        // K_kj = s/r [ (c2 delta_kj + 2 d_k d_j / r^2) drdm + sgn c2 (m_j d_k - m_k d_j)/r ]
        // (the 3D form below with one power of r less and 2 for 3)
        const T mx = KID == EL_TRAC2 ? nsx : nox;
        const T my = KID == EL_TRAC2 ? nsy : noy;
        const T ir2 = ir * ir;
        const T drdm = (dx * mx + dy * my) * ir;
        const T dv = dx * v[0] + dy * v[1];
        const T mv = mx * v[0] + my * v[1];
        const T a = T(2) * dv * ir2;
        const T sg = KID == EL_TRAC2 ? T(-1) : T(1);
        const T b = sg * c2 * ir;
        const T s = (KID == EL_TRAC2 ? T(-1) : T(1)) * ir;
        if (!TRANS) {
            u[0] += s * (drdm * (c2 * v[0] + dx * a) + b * (dx * mv - mx * dv));
            u[1] += s * (drdm * (c2 * v[1] + dy * a) + b * (dy * mv - my * dv));
        } else {
            u[0] += s * (drdm * (c2 * v[0] + dx * a) + b * (mx * dv - dx * mv));
            u[1] += s * (drdm * (c2 * v[1] + dy * a) + b * (my * dv - dy * mv));
        }
    } else if (KID == EL_TRAC || KID == EL_ADJ) {
        // K_kj = s/r^2 [ (c2 delta_kj + 3 d_k d_j / r^2) drdm + sgn c2 (m_j d_k - m_k d_j)/r ]
        // with m = n_y, s = -1, sgn = -1 for the traction kernel and m = n_x,
        // s = +1, sgn = +1 for the adjoint traction kernel.
        const T mx = KID == EL_TRAC ? nsx : nox;
        const T my = KID == EL_TRAC ? nsy : noy;
        const T mz = KID == EL_TRAC ? nsz : noz;
        const T ir2 = ir * ir;
        const T dm = dx * mx + dy * my + dz * mz;
        const T drdm = dm * ir;
        const T dv = dx * v[0] + dy * v[1] + dz * v[2];
        const T mv = mx * v[0] + my * v[1] + mz * v[2];
        const T a = T(3) * dv * ir2;
        // term2 contraction: sum_j (m_j d_k - m_k d_j) v_j = d_k mv - m_k dv; transposed:
        // sum_k (m_j d_k - m_k d_j) v_k = m_j dv - d_j mv.
        const T sg = KID == EL_TRAC ? T(-1) : T(1);
        const T b = sg * c2 * ir;
        const T s = (KID == EL_TRAC ? T(-1) : T(1)) * ir2;
        if (!TRANS) {
            u[0] += s * (drdm * (c2 * v[0] + dx * a) + b * (dx * mv - mx * dv));
            u[1] += s * (drdm * (c2 * v[1] + dy * a) + b * (dy * mv - my * dv));
            u[2] += s * (drdm * (c2 * v[2] + dz * a) + b * (dz * mv - mz * dv));
        } else {
            u[0] += s * (drdm * (c2 * v[0] + dx * a) + b * (mx * dv - dx * mv));
            u[1] += s * (drdm * (c2 * v[1] + dy * a) + b * (my * dv - dy * mv));
            u[2] += s * (drdm * (c2 * v[2] + dz * a) + b * (mz * dv - dz * mv));
        }
    }
}

// Full tensor (row-major R x C, constant included) for operator assembly.
template <typename T>
__device__ __forceinline__ void kernel_tensor(int kid, T dx, T dy, T dz, T nox, T noy, T noz,
                                              T nsx, T nsy, T nsz, const KParams& p, T* out)
{
    const int R = kernel_dim(kid);
    const T r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < T(1e-12)) {
        for (int i = 0; i < R * R; i++) out[i] = 0;
        return;
    }
    const T r = sqrt(r2);
    const T d[3] = {dx, dy, dz};
    if (kid == LAP_S) {
        out[0] = T(p.scale) / r;
    } else if (kid == LAP_D) {
        out[0] = T(p.scale) * (nsx * dx + nsy * dy + nsz * dz) / (r2 * r);
    } else if (kid == IDENT) {
        out[0] = 1;
    } else if (kid == EL_DISP) {
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++)
                out[3 * k + j] = (T(p.scale) / r) * (T(p.c2) * (k == j) + d[k] * d[j] / r2);
    } else if (kid == EL_HYP) {
        T H[9];
        hyp_tensor<T>(dx, dy, dz, r2, T(1) / r, nox, noy, noz, nsx, nsy, nsz, T(p.c2), H);
        for (int i = 0; i < 9; i++) out[i] = T(p.scale) * H[i];
    } else {
        const bool trac = kid == EL_TRAC;
        const T m[3] = {trac ? nsx : nox, trac ? nsy : noy, trac ? nsz : noz};
        const T drdm = (d[0] * m[0] + d[1] * m[1] + d[2] * m[2]) / r;
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++) {
                const T term1 = T(p.c2) * (k == j) + T(3) * d[k] * d[j] / r2;
                const T term2 = T(p.c2) * (m[j] * d[k] - m[k] * d[j]) / r;
                out[3 * k + j] = trac ? -(T(p.scale) / r2) * (term1 * drdm - term2)
                                      : (T(p.scale) / r2) * (term1 * drdm + term2);
            }
    }
}

// Full 2D tensor (row-major R x C, constant included).
template <typename T>
__device__ __forceinline__ void kernel_tensor_2d(int kid, T dx, T dy, T nox, T noy, T nsx, T nsy,
                                                 const KParams& p, T* out)
{
    const int R = kernel_dim(kid);
    const T r2 = dx * dx + dy * dy;
    if (r2 < T(1e-12)) {
        for (int i = 0; i < R * R; i++) out[i] = 0;
        return;
    }
    const T r = sqrt(r2);
    const T d[2] = {dx, dy};
    const T sc = T(p.scale), c2 = T(p.c2);
    if (kid == LAP_S2) {
        out[0] = sc * dev_log<T>(r);
    } else if (kid == LAP_D2) {
        out[0] = sc * (nsx * dx + nsy * dy) / r2;
    } else if (kid == LAP_H2) {
        const T dn = nsx * dx + nsy * dy, dm = nox * dx + noy * dy;
        out[0] = sc * (-(nox * nsx + noy * nsy) / r2 + T(2) * dn * dm / (r2 * r2));
    } else if (kid == IDENT2) {
        out[0] = 1;
    } else if (kid == EL_DISP2) {
        const T lr = dev_log<T>(r);
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++)
                out[2 * k + j] = sc * (-c2 * T(k == j) * lr + d[k] * d[j] / r2);
    } else if (kid == EL_HYP2) {
        T H[4];
        hyp_tensor_2d<T>(dx, dy, T(1) / r, nox, noy, nsx, nsy, c2, H);
        for (int i = 0; i < 4; i++) out[i] = sc * H[i];
    } else {
        const bool trac = kid == EL_TRAC2;
        const T m[2] = {trac ? nsx : nox, trac ? nsy : noy};
        const T drdm = (d[0] * m[0] + d[1] * m[1]) / r;
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++) {
                const T term1 = c2 * T(k == j) + T(2) * d[k] * d[j] / r2;
                const T term2 = c2 * (m[j] * d[k] - m[k] * d[j]) / r;
                out[2 * k + j] = trac ? -(sc / r) * (term1 * drdm - term2)
                                      : (sc / r) * (term1 * drdm + term2);
            }
    }
}

// kernel_tensor for any kernel id (3D or 2D); 2D ids read x and y only.
template <typename T>
__device__ __forceinline__ void kernel_tensor_any(int kid, T dx, T dy, T dz, T nox, T noy, T noz,
                                                  T nsx, T nsy, T nsz, const KParams& p, T* out)
{
    if (kernel_space_dim(kid) == 2) kernel_tensor_2d<T>(kid, dx, dy, nox, noy, nsx, nsy, p, out);
    else kernel_tensor<T>(kid, dx, dy, dz, nox, noy, noz, nsx, nsy, nsz, p, out);
}

}  // namespace tbem
