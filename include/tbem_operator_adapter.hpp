// tbem_operator_adapter.hpp -- C++ adapters that put the GB300 library behind
// the reference's own interfaces.  A maintainer of tbenthompson/3bem adds this
// header to the reference tree (it includes the reference's operator.h,
// fmm.h, nbody_operator.h and sparse_operator.h) and links -ltbem_gpu.
//
//   GpuFMMOperator<R>  an OperatorI (cpp/operator.h:14-19) over the FMM handle;
//                      IntegralOperator takes it as its farfield
//                      (cpp/integral_operator.h:31, built at :82-88)
//   gpu_nearfield      a SparseOperator (cpp/sparse_operator.h:44-83) from the
//                      GPU nearfield construction, for make_nearfield_operator /
//                      make_farfield_correction_operator
//                      (cpp/integral_operator.h:72-76)
#pragma once
#include <memory>
#include <stdexcept>
#include <vector>

#include "fmm.h"
#include "nbody_operator.h"
#include "operator.h"
#include "sparse_operator.h"
#include "tbem_gpu.h"

namespace tbem {

template <size_t R>
struct GpuFMMOperator : public OperatorI {
    TbemFmm* h = nullptr;
    GpuFMMOperator(int kernel_id, const double* params, const NBodyData<3>& d,
                   const FMMConfig& c, int precision = TBEM_PRECISION_FP64) {
        TbemFmmConfig cfg{c.mac, (long)c.order, (long)c.min_pts_per_cell, c.d,
                          c.account_for_small_cells};
        TbemGpuOptions opt; tbem_default_options(&opt); opt.precision = precision;
        int rc = tbem_fmm_create(kernel_id, params,
            &d.obs_locs[0][0], &d.obs_normals[0][0], (long)d.obs_locs.size(),
            &d.src_locs[0][0], &d.src_normals[0][0], d.src_weights.data(),
            (long)d.src_locs.size(), &cfg, &opt, &h);
        if (rc != TBEM_OK) throw std::runtime_error(tbem_last_error());
    }
    explicit GpuFMMOperator(TbemFmm* handle) : h(handle) {}
    ~GpuFMMOperator() { tbem_fmm_destroy(h); }
    size_t n_rows() const override { return (size_t)tbem_fmm_n_rows(h); }
    size_t n_cols() const override { return (size_t)tbem_fmm_n_cols(h); }
    std::vector<double> apply(const std::vector<double>& x) const override {
        std::vector<double> y(n_rows());
        if (tbem_fmm_apply(h, x.data(), y.data(), 1, nullptr) != TBEM_OK)
            throw std::runtime_error(tbem_last_error());
        return y;
    }
    std::unique_ptr<OperatorI> clone() const override {
        TbemFmm* c = nullptr;
        if (tbem_fmm_clone(h, &c) != TBEM_OK) throw std::runtime_error(tbem_last_error());
        return std::unique_ptr<OperatorI>(new GpuFMMOperator<R>(c));
    }
};

// vertices [n][3], facets [m][3] (indices), the same mesh as obs, src and all
inline SparseOperator gpu_nearfield(int kernel_id, const double* params,
    const std::vector<double>& vertices, const std::vector<long>& facets,
    int strategy /* TBEM_QUAD_SINH or TBEM_QUAD_ADAPTIVE */, double near_tol,
    long sinh_order, long obs_near_order, long obs_far_order, long src_far_order,
    long n_singular_steps, double far_threshold, int which /* 0 near, 1 correction */)
{
    TbemIntegrator m{strategy, near_tol, sinh_order, obs_near_order, obs_far_order,
                     src_far_order, n_singular_steps, far_threshold};
    const long nv = (long)vertices.size() / 3, nf = (long)facets.size() / 3;
    TbemCsr* h = nullptr;
    if (tbem_nearfield_create(kernel_id, params, vertices.data(), nv, facets.data(), nf,
                              facets.data(), nf, facets.data(), nf, &m, which, &h) != TBEM_OK)
        throw std::runtime_error(tbem_last_error());
    long nr = 0, nc = 0;
    tbem_csr_shape(h, &nr, &nc);
    const long nnz = tbem_csr_nnz(h);
    std::vector<double> v(nnz);
    std::vector<long> c(nnz), r(nr + 1);
    tbem_csr_download(h, v.data(), c.data(), r.data());
    tbem_csr_destroy(h);
    return SparseOperator(nr, nc, v, std::vector<size_t>(c.begin(), c.end()),
                          std::vector<size_t>(r.begin(), r.end()));
}

}  // namespace tbem
