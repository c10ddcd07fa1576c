// Direct FP64 N-body sum on the GPU and the CSR operator.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "handle.h"
#include "nearfield.h"

namespace {

struct Staged {
    const double* p = nullptr;
    tbem::DBuf<double> own;
};

bool is_device(const void* p)
{
    cudaPointerAttributes a{};
    bool dev = p && cudaPointerGetAttributes(&a, p) == cudaSuccess &&
               (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    return dev;
}

// Device view of a caller array (copied in when it is host memory).
void stage(Staged& s, const double* p, size_t n, cudaStream_t st)
{
    if (n == 0) { s.p = nullptr; return; }
    if (is_device(p)) { s.p = p; return; }
    s.own.alloc(n);
    TBEM_CK(cudaMemcpyAsync(s.own.p, p, n * sizeof(double), cudaMemcpyHostToDevice, st));
    s.p = s.own.p;
}

__global__ void widen_kernel(const double* in, double* out, long n)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        out[3 * i] = in[2 * i];
        out[3 * i + 1] = in[2 * i + 1];
        out[3 * i + 2] = 0.0;
    }
}

// Device view of caller points [n][sdim] as [n][3] (2D points get z = 0).
void stage_points(Staged& s, const double* p, long n, int sdim, cudaStream_t st)
{
    if (sdim == 3) {
        stage(s, p, 3 * (size_t)n, st);
        return;
    }
    Staged raw;
    stage(raw, p, 2 * (size_t)n, st);
    s.own.alloc(3 * (size_t)n);
    widen_kernel<<<(unsigned)std::max<long>(1, std::min<long>((n + 255) / 256, 9728)), 256, 0, st>>>(
        raw.p, s.own.p, n);
    TBEM_CK(cudaGetLastError());
    // raw's own buffer (if any) is freed on return: finish the copy first
    TBEM_CK(cudaStreamSynchronize(st));
    s.p = s.own.p;
}

__global__ void weight_kernel(const double* x, const double* w, double* s, long N, long total)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x)
        s[t] = w[t % N] * x[t];
}

// y = A x (add = 0) or y += A x (add = 1).  L lanes per row (L chosen per
// matrix from its mean row length): a lane takes the row's entries k = b +
// lane, + L, ..., CSR_UNROLL of them per step, loading all their values and
// columns before any gather of x, so every lane keeps CSR_UNROLL independent
// loads in flight (the gather x[col[k]] waits on the column load: with one
// entry per lane per step the SpMV was latency-bound at a third of the
// copy bandwidth); the L partial sums meet in shuffles.
constexpr int CSR_UNROLL = 4, CSR_THREADS = 256;

template <int L>
__global__ void __launch_bounds__(CSR_THREADS)
csr_kernel(const long* __restrict__ rowptr, const long* __restrict__ col, const double* __restrict__ val,
           const double* __restrict__ x, double* y, long n_rows, long n_cols, int nrhs, int add)
{
    const long row = ((long)blockIdx.x * blockDim.x + threadIdx.x) / L;
    const int lane = threadIdx.x % L;
    if (row >= n_rows) return;  // whole L-lane groups leave together
    const unsigned mask = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << ((threadIdx.x % 32) / L * L));
    const long b = rowptr[row], e = rowptr[row + 1];
    for (int r = 0; r < nrhs; r++) {
        const double* xr = x + (long)r * n_cols;
        double acc = 0.0;
        for (long k0 = b + lane; k0 < e; k0 += (long)CSR_UNROLL * L) {
            double v[CSR_UNROLL];
            long c[CSR_UNROLL];
#pragma unroll
            for (int u = 0; u < CSR_UNROLL; u++) {
                const long k = k0 + (long)u * L;
                v[u] = k < e ? val[k] : 0.0;
                c[u] = k < e ? col[k] : -1;
            }
#pragma unroll
            for (int u = 0; u < CSR_UNROLL; u++)
                if (c[u] >= 0) acc += v[u] * xr[c[u]];
        }
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(mask, acc, o);
        if (lane == 0) {
            double* d = y + (long)r * n_rows + row;
            *d = add ? *d + acc : acc;
        }
    }
}

// FMA-rate microbenchmark: FMA_CHAINS independent chains a = a * b + c per
// thread, FMA_UNROLL steps per iteration.  b < 1 keeps the values bounded;
// the store happens only for a sum no chain reaches, so nothing is written
// while the compiler must still compute every chain.
constexpr int FMA_CHAINS = 8, FMA_UNROLL = 16, FMA_THREADS = 256;

template <typename T>
__global__ void __launch_bounds__(FMA_THREADS) fma_peak_kernel(T* out, int iters, T b, T c)
{
    T a[FMA_CHAINS];
#pragma unroll
    for (int i = 0; i < FMA_CHAINS; i++) a[i] = T(threadIdx.x + i) * T(1e-3);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < FMA_UNROLL; k++)
#pragma unroll
            for (int i = 0; i < FMA_CHAINS; i++) a[i] = fma(a[i], b, c);
    }
    T s = T(0);
#pragma unroll
    for (int i = 0; i < FMA_CHAINS; i++) s += a[i];
    if (s == T(-1)) out[(long)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
double fma_peak(int device)
{
    using namespace tbem;
    DeviceGuard guard(device);
    int sms = 0, threads = 0;
    TBEM_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    TBEM_CK(cudaDeviceGetAttribute(&threads, cudaDevAttrMaxThreadsPerMultiProcessor, device));
    const int blocks = sms * std::max(threads / FMA_THREADS, 1);
    const double per_iter = 2.0 * FMA_CHAINS * FMA_UNROLL * (double)blocks * FMA_THREADS;
    DBuf<T> out;
    out.alloc((size_t)blocks * FMA_THREADS);
    cudaStream_t s;
    TBEM_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    TBEM_CK(cudaEventCreate(&e0));
    TBEM_CK(cudaEventCreate(&e1));
    // size the run to ~10 ms from a short first run
    int iters = 64;
    double best = 0.0;
    for (int run = 0; run < 5; run++) {
        TBEM_CK(cudaEventRecord(e0, s));
        fma_peak_kernel<T><<<blocks, FMA_THREADS, 0, s>>>(out.p, iters, T(0.999), T(1e-3));
        TBEM_CK(cudaGetLastError());
        TBEM_CK(cudaEventRecord(e1, s));
        TBEM_CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        TBEM_CK(cudaEventElapsedTime(&ms, e0, e1));
        const double tf = per_iter * iters / (ms * 1e-3) / 1e12;
        if (run >= 2) best = std::max(best, tf);  // runs 0-1: sizing and warm-up
        if (run == 0) iters = std::max(1, (int)std::min(1e8, iters * 10.0 / std::max((double)ms, 1e-3)));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    return best;
}
}  // namespace

struct TbemCsr {
    long n_rows = 0, n_cols = 0, nnz = 0;
    int lanes = 32;  // lanes per row of the SpMV kernel
    tbem::DBuf<long> rowptr, col;
    tbem::DBuf<double> val;
};

namespace {
// y (+)= A x on stream s (A non-empty)
void csr_launch(const TbemCsr* A, const double* x, double* y, int nrhs, int add, cudaStream_t s)
{
    const int L = A->lanes;
    const unsigned blocks = (unsigned)((A->n_rows * L + CSR_THREADS - 1) / CSR_THREADS);
    auto go = [&](auto kern) {
        kern<<<blocks, CSR_THREADS, 0, s>>>(A->rowptr.p, A->col.p, A->val.p, x, y, A->n_rows, A->n_cols,
                                            nrhs, add);
    };
    if (L == 4) go(csr_kernel<4>);
    else if (L == 8) go(csr_kernel<8>);
    else if (L == 16) go(csr_kernel<16>);
    else go(csr_kernel<32>);
    TBEM_CK(cudaGetLastError());
}
}  // namespace

extern "C" {

int tbem_direct_apply(int kernel, const double* kernel_params, const double* obs_locs,
                      const double* obs_normals, long n_obs, const double* src_locs,
                      const double* src_normals, const double* src_weights, long n_src,
                      const double* x, double* y, int n_rhs, void* stream)
{
    using namespace tbem;
    try {
        if (!kernel_valid(kernel) || n_obs < 0 || n_src < 0 || n_rhs <= 0 || !y)
            throw Error(TBEM_ERR_ARG, "bad argument");
        if (n_src > (long)INT32_MAX) throw Error(TBEM_ERR_ARG, "too many sources");
        if (n_obs > 0 && n_src > 0 && (!obs_locs || !obs_normals || !src_locs || !src_normals ||
                                       !src_weights || !x))
            throw Error(TBEM_ERR_ARG, "null point or input array");
        const int R = kernel_dim(kernel);
        const int sdim = kernel_space_dim(kernel);
        const double mu = (kernel_params && R > 1) ? kernel_params[0] : 1.0;
        const double nu = (kernel_params && R > 1) ? kernel_params[1] : 0.25;
        const KParams kp = make_kparams(kernel, mu, nu);
        cudaStream_t s = (cudaStream_t)stream;
        const bool y_dev = is_device(y);
        const size_t ny = (size_t)R * n_obs * n_rhs;
        if (n_obs == 0) return TBEM_OK;
        DBuf<double> ybuf;
        double* yd = y;
        if (!y_dev) { ybuf.alloc(ny); yd = ybuf.p; }
        if (n_src == 0) {
            TBEM_CK(cudaMemsetAsync(yd, 0, ny * sizeof(double), s));
        } else {
            Staged ol, on, sl, sn, sw, xs;
            stage_points(ol, obs_locs, n_obs, sdim, s);
            stage_points(on, obs_normals, n_obs, sdim, s);
            stage_points(sl, src_locs, n_src, sdim, s);
            stage_points(sn, src_normals, n_src, sdim, s);
            stage(sw, src_weights, n_src, s);
            stage(xs, x, (size_t)R * n_src * n_rhs, s);
            DBuf<double> str;
            str.alloc((size_t)R * n_src * n_rhs);
            const long tot = (long)R * n_src * n_rhs;
            weight_kernel<<<std::max<long>(1, std::min<long>((tot + 255) / 256, 9728)), 256, 0, s>>>(xs.p, sw.p, str.p, n_src, tot);
            TBEM_CK(cudaGetLastError());
            // tasks: chunks of observation points against all sources
            TaskSet ts;
            const int chunk = 1024;
            double org[3] = {0, 0, 0};
            for (long b = 0; b < n_obs; b += chunk)
                ts.add(b, (int)std::min<long>(chunk, n_obs - b), org, {{0L, (int)n_src}}, EVAL_THREADS / 4);
            ts.upload();
            EvalArgs<double> a{};
            ts.fill(a);
            a.t_xyz = ol.p;
            a.t_nrm = on.p;
            a.s_xyz = sl.p;
            a.s_nrm = sn.p;
            a.s_str = str.p;
            a.s_n = n_src;
            a.y = yd;
            a.y_n = n_obs;
            a.nrhs = n_rhs;
            a.add = 0;
            a.c2 = kp.c2;
            a.scale = kp.scale;
            EvalLaunch L{kernel, false, false, false, ts.n_items()};
            for (int r0 = 0; r0 < n_rhs; r0 += (n_rhs - r0 > 1 ? EVAL_NR : 1)) {
                a.rhs0 = r0;
                TBEM_CK(launch_eval<double>(L, a, s));
            }
        }
        if (!y_dev) TBEM_CK(cudaMemcpyAsync(y, yd, ny * sizeof(double), cudaMemcpyDeviceToHost, s));
        TBEM_CK(cudaStreamSynchronize(s));
        return TBEM_OK;
    } catch (...) {
        return tbem::api_status();
    }
}

int tbem_csr_create(long n_rows, long n_cols, const double* values, const long* column_indices,
                    const long* row_ptrs, TbemCsr** out)
{
    using namespace tbem;
    if (!out || n_rows < 0 || n_cols < 0 || !row_ptrs) return TBEM_ERR_ARG;
    *out = nullptr;
    try {
        if (row_ptrs[0] != 0) throw Error(TBEM_ERR_ARG, "row_ptrs[0] must be 0");
        for (long i = 0; i < n_rows; i++)
            if (row_ptrs[i + 1] < row_ptrs[i]) throw Error(TBEM_ERR_ARG, "row_ptrs must not decrease");
        const long nnz = row_ptrs[n_rows];
        if (nnz > 0 && (!values || !column_indices)) throw Error(TBEM_ERR_ARG, "null values");
        // column check on all host cores, in blocks (one flag per block)
        const long block = 1 << 20, n_blocks = (nnz + block - 1) / block;
        std::vector<char> bad(n_blocks, 0);
        nf::parallel_for(
            n_blocks,
            [&](long b) {
                for (long k = b * block; k < std::min(nnz, (b + 1) * block); k++)
                    if (column_indices[k] < 0 || column_indices[k] >= n_cols) bad[b] = 1;
            },
            1);
        if (std::find(bad.begin(), bad.end(), 1) != bad.end())
            throw Error(TBEM_ERR_ARG, "column index out of range");
        auto h = std::make_unique<TbemCsr>();
        h->n_rows = n_rows;
        h->n_cols = n_cols;
        h->nnz = nnz;
        // lanes per row: the fewest that take a mean row in one unrolled step
        const double mean = n_rows > 0 ? (double)nnz / (double)n_rows : 0.0;
        h->lanes = mean <= 4 * CSR_UNROLL ? 4 : mean <= 8 * CSR_UNROLL ? 8 : mean <= 16 * CSR_UNROLL ? 16 : 32;
        h->rowptr.upload(row_ptrs, (size_t)n_rows + 1);
        if (nnz > 0) {
            h->col.upload(column_indices, (size_t)nnz);
            h->val.upload(values, (size_t)nnz);
        }
        *out = h.release();
        return TBEM_OK;
    } catch (...) {
        return tbem::api_status();
    }
}

int tbem_csr_apply(TbemCsr* h, const double* x, double* y, int n_rhs, void* stream)
{
    using namespace tbem;
    if (!h || !y || n_rhs <= 0 || (!x && h->n_cols > 0)) {
        tbem::set_last_error("null argument or n_rhs <= 0");
        return TBEM_ERR_ARG;
    }
    try {
        cudaStream_t s = (cudaStream_t)stream;
        if (h->n_rows == 0) return TBEM_OK;
        const size_t ny = (size_t)h->n_rows * n_rhs;
        const bool y_dev = is_device(y);
        DBuf<double> ybuf;
        double* yd = y;
        if (!y_dev) { ybuf.alloc(ny); yd = ybuf.p; }
        if (h->nnz == 0) {
            TBEM_CK(cudaMemsetAsync(yd, 0, ny * sizeof(double), s));
        } else {
            Staged xs;
            stage(xs, x, (size_t)h->n_cols * n_rhs, s);
            csr_launch(h, xs.p, yd, n_rhs, 0, s);
        }
        if (!y_dev) TBEM_CK(cudaMemcpyAsync(y, yd, ny * sizeof(double), cudaMemcpyDeviceToHost, s));
        TBEM_CK(cudaStreamSynchronize(s));
        return TBEM_OK;
    } catch (...) {
        return tbem::api_status();
    }
}

long tbem_csr_nnz(const TbemCsr* h) { return h ? h->nnz : TBEM_ERR_ARG; }

int tbem_csr_shape(const TbemCsr* h, long* n_rows, long* n_cols)
{
    if (!h) return TBEM_ERR_ARG;
    if (n_rows) *n_rows = h->n_rows;
    if (n_cols) *n_cols = h->n_cols;
    return TBEM_OK;
}

int tbem_csr_download(const TbemCsr* h, double* values, long* column_indices, long* row_ptrs)
{
    using namespace tbem;
    if (!h) return TBEM_ERR_ARG;
    try {
        if (row_ptrs)
            TBEM_CK(cudaMemcpy(row_ptrs, h->rowptr.p, sizeof(long) * (h->n_rows + 1), cudaMemcpyDeviceToHost));
        if (h->nnz > 0 && values)
            TBEM_CK(cudaMemcpy(values, h->val.p, sizeof(double) * h->nnz, cudaMemcpyDeviceToHost));
        if (h->nnz > 0 && column_indices)
            TBEM_CK(cudaMemcpy(column_indices, h->col.p, sizeof(long) * h->nnz, cudaMemcpyDeviceToHost));
        return TBEM_OK;
    } catch (...) {
        return tbem::api_status();
    }
}

void tbem_csr_destroy(TbemCsr* h) { delete h; }


// ---- IntegralOperator: y = G (F (I x)) + N x + C x on the device -------------

}  // extern "C"

struct TbemIntegral {
    TbemCsr *near = nullptr, *corr = nullptr, *galerkin = nullptr, *interp = nullptr;
    TbemFmm* far = nullptr;
    long n_rows = 0, n_cols = 0;
    tbem::DBuf<double> xi, xf, yf, yo;  // I x, F (I x), staged output
};

namespace {
void csr_into(const TbemCsr* A, const double* x, double* y, int nrhs, int add, cudaStream_t s)
{
    if (A->n_rows == 0) return;
    if (A->nnz == 0) {
        if (!add) TBEM_CK(cudaMemsetAsync(y, 0, sizeof(double) * A->n_rows * nrhs, s));
        return;
    }
    csr_launch(A, x, y, nrhs, add, s);
}
}  // namespace

extern "C" {

int tbem_integral_create(TbemCsr* nearfield, TbemCsr* correction, TbemCsr* galerkin,
                         TbemFmm* farfield, TbemCsr* interp, TbemIntegral** out)
{
    if (!out) return TBEM_ERR_ARG;
    *out = nullptr;
    if (!nearfield || !correction || !galerkin || !farfield || !interp) {
        tbem::set_last_error("null operator");
        return TBEM_ERR_ARG;
    }
    const long fr = tbem_fmm_n_rows(farfield), fc = tbem_fmm_n_cols(farfield);
    const long n = nearfield->n_rows, m = nearfield->n_cols;
    if (correction->n_rows != n || correction->n_cols != m || galerkin->n_rows != n ||
        galerkin->n_cols != fr || interp->n_rows != fc || interp->n_cols != m) {
        tbem::set_last_error("operator shapes do not chain: G (n x F rows), F, I (F cols x m), N and C (n x m)");
        return TBEM_ERR_ARG;
    }
    TbemIntegral* h = new TbemIntegral();
    h->near = nearfield;
    h->corr = correction;
    h->galerkin = galerkin;
    h->far = farfield;
    h->interp = interp;
    h->n_rows = n;
    h->n_cols = m;
    *out = h;
    return TBEM_OK;
}

int tbem_integral_apply(TbemIntegral* h, const double* x, double* y, int n_rhs, void* stream)
{
    using namespace tbem;
    if (!h || !y || n_rhs <= 0 || (!x && h->n_cols > 0)) {
        set_last_error("null argument or n_rhs <= 0");
        return TBEM_ERR_ARG;
    }
    try {
        // one stream for the whole chain: the caller's, else the farfield's own
        // (the FMM apply would otherwise run on that one, unordered with the
        // sparse steps)
        cudaStream_t s = stream ? (cudaStream_t)stream : h->far->plan.stream;
        if (h->n_rows == 0) return TBEM_OK;
        const size_t ny = (size_t)h->n_rows * n_rhs;
        const bool y_dev = is_device(y);
        double* yd = y;
        if (!y_dev) {
            h->yo.ensure(ny);
            yd = h->yo.p;
        }
        Staged xs;
        stage(xs, x, (size_t)h->n_cols * n_rhs, s);
        const long fr = tbem_fmm_n_rows(h->far), fc = tbem_fmm_n_cols(h->far);
        h->xi.ensure(std::max<size_t>((size_t)fc * n_rhs, 1));
        h->xf.ensure(std::max<size_t>((size_t)fr * n_rhs, 1));
        csr_into(h->interp, xs.p, h->xi.p, n_rhs, 0, s);               // I x
        h->far->plan.apply(h->xi.p, h->xf.p, n_rhs, s, false);        // F (I x)
        csr_into(h->galerkin, h->xf.p, yd, n_rhs, 0, s);               // G F I x
        csr_into(h->near, xs.p, yd, n_rhs, 1, s);                      // + N x
        csr_into(h->corr, xs.p, yd, n_rhs, 1, s);                      // + C x
        if (!y_dev) TBEM_CK(cudaMemcpyAsync(y, yd, ny * sizeof(double), cudaMemcpyDeviceToHost, s));
        TBEM_CK(cudaStreamSynchronize(s));
        return TBEM_OK;
    } catch (...) {
        return api_status();
    }
}

long tbem_integral_n_rows(const TbemIntegral* h) { return h ? h->n_rows : TBEM_ERR_ARG; }
long tbem_integral_n_cols(const TbemIntegral* h) { return h ? h->n_cols : TBEM_ERR_ARG; }
void tbem_integral_destroy(TbemIntegral* h) { delete h; }

int tbem_setup_cache_clear(void)
{
    tbem::clear_setup_cache();
    return TBEM_OK;
}

int tbem_fma_peak(int device, int fp64, double* tflops)
{
    using namespace tbem;
    if (!tflops) {
        set_last_error("null output");
        return TBEM_ERR_ARG;
    }
    try {
        *tflops = fp64 ? fma_peak<double>(device) : fma_peak<float>(device);
        return TBEM_OK;
    } catch (...) {
        return api_status();
    }
}

}  // extern "C"
