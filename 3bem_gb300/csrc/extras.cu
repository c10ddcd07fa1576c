// Direct FP64 N-body sum on the GPU and the CSR operator.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "plan.h"

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

__global__ void weight_kernel(const double* x, const double* w, double* s, long N, long total)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x)
        s[t] = w[t % N] * x[t];
}

__global__ void csr_kernel(const long* rowptr, const long* col, const double* val, const double* x,
                           double* y, long n_rows, long n_cols, int nrhs)
{
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x % 32;
    if (warp >= n_rows) return;
    const long b = rowptr[warp], e = rowptr[warp + 1];
    for (int r = 0; r < nrhs; r++) {
        const double* xr = x + (long)r * n_cols;
        double acc = 0.0;
        for (long k = b + lane; k < e; k += 32) acc += val[k] * xr[col[k]];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) y[(long)r * n_rows + warp] = acc;
    }
}
}  // namespace

struct TbemCsr {
    long n_rows = 0, n_cols = 0, nnz = 0;
    tbem::DBuf<long> rowptr, col;
    tbem::DBuf<double> val;
};

extern "C" {

int tbem_direct_apply(int kernel, const double* kernel_params, const double* obs_locs,
                      const double* obs_normals, long n_obs, const double* src_locs,
                      const double* src_normals, const double* src_weights, long n_src,
                      const double* x, double* y, int n_rhs, void* stream)
{
    using namespace tbem;
    try {
        if (kernel < 0 || kernel > 5 || n_obs < 0 || n_src < 0 || n_rhs <= 0 || !y)
            throw Error(TBEM_ERR_ARG, "bad argument");
        const int R = kernel_dim(kernel);
        const double mu = (kernel_params && R == 3) ? kernel_params[0] : 1.0;
        const double nu = (kernel_params && R == 3) ? kernel_params[1] : 0.25;
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
            stage(ol, obs_locs, 3 * n_obs, s);
            stage(on, obs_normals, 3 * n_obs, s);
            stage(sl, src_locs, 3 * n_src, s);
            stage(sn, src_normals, 3 * n_src, s);
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
            if (n_src > (long)INT32_MAX) throw Error(TBEM_ERR_ARG, "too many sources");
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
    } catch (const tbem::Error& e) {
        tbem::set_last_error(e.what());
        return e.code;
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
        for (long k = 0; k < nnz; k++)
            if (column_indices[k] < 0 || column_indices[k] >= n_cols)
                throw Error(TBEM_ERR_ARG, "column index out of range");
        auto h = new TbemCsr();
        h->n_rows = n_rows;
        h->n_cols = n_cols;
        h->nnz = nnz;
        h->rowptr.upload(std::vector<long>(row_ptrs, row_ptrs + n_rows + 1));
        if (nnz > 0) {
            h->col.upload(std::vector<long>(column_indices, column_indices + nnz));
            h->val.upload(std::vector<double>(values, values + nnz));
        }
        *out = h;
        return TBEM_OK;
    } catch (const tbem::Error& e) {
        tbem::set_last_error(e.what());
        return e.code;
    }
}

int tbem_csr_apply(TbemCsr* h, const double* x, double* y, int n_rhs, void* stream)
{
    using namespace tbem;
    if (!h || !y || n_rhs <= 0) return TBEM_ERR_ARG;
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
            const long threads = h->n_rows * 32;
            csr_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(h->rowptr.p, h->col.p, h->val.p, xs.p, yd, h->n_rows, h->n_cols, n_rhs);
            TBEM_CK(cudaGetLastError());
        }
        if (!y_dev) TBEM_CK(cudaMemcpyAsync(y, yd, ny * sizeof(double), cudaMemcpyDeviceToHost, s));
        TBEM_CK(cudaStreamSynchronize(s));
        return TBEM_OK;
    } catch (const tbem::Error& e) {
        tbem::set_last_error(e.what());
        return e.code;
    }
}

long tbem_csr_nnz(const TbemCsr* h) { return h ? h->nnz : TBEM_ERR_ARG; }

void tbem_csr_destroy(TbemCsr* h) { delete h; }

}  // extern "C"
