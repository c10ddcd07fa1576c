// Test driver: the product's host plan of a nearfield / farfield-correction
// matrix (3bem_gb300/csrc/nearfield_host.cpp: galerkin_obs_points,
// plan_terms, assemble_csr) with the far evaluations done here on the CPU by
// the oracle's kernels, so that tests/test_nearfield_host.py can compare the
// matrix layout (both matrices) and the correction matrix's values with the
// reference's on the CPU.  The product evaluates the same items on the GPU.
//
// stdin: kernel mu nu dim obs_order far_threshold n_steps src_far_order which
//        n_vertices, vertices [n][3], n_facets, facets [n][dim]
// stdout: n_rows n_cols nnz, then row_ptrs, cols, values (one line each);
//         values are the correction matrix's for which = 1, zeros otherwise.
#include <cstdio>
#include <vector>

#include "nearfield.h"

extern "C" int oracle_kernel(int kernel, double mu, double nu, const double* obs, const double* src,
                             const double* nobs, const double* nsrc, double* out);

using namespace tbem::nf;

int main()
{
    int kernel, dim, order, n_steps, src_far_order, which;
    double mu, nu, far;
    if (scanf("%d %lf %lf %d %d %lf %d %d %d", &kernel, &mu, &nu, &dim, &order, &far, &n_steps,
              &src_far_order, &which) != 9)
        return 1;
    long nv, nf;
    if (scanf("%ld", &nv) != 1) return 1;
    std::vector<V3> v(nv);
    for (auto& x : v)
        if (scanf("%lf %lf %lf", &x.x[0], &x.x[1], &x.x[2]) != 3) return 1;
    if (scanf("%ld", &nf) != 1) return 1;
    std::vector<Facet> fac(nf);
    for (auto& f : fac)
        for (int q = 0; q < dim; q++) {
            long k;
            if (scanf("%ld", &k) != 1) return 1;
            f.c[q] = v[k];
        }
    const FacetSet set(fac, dim);
    const ObsPoints pts = galerkin_obs_points(fac, set, order, dim);
    const TermPlan tp = plan_terms(pts, fac, set, far, n_steps, dim, which == 1);
    double probe[9];
    const double z[3] = {0, 0, 0}, one[3] = {1, 0, 0};
    const int RR = oracle_kernel(kernel, mu, nu, z, one, one, one, probe);
    const int R = RR == 9 ? 3 : RR == 4 ? 2 : 1;
    const int E = dim * R * R;
    std::vector<double> ivals(tp.i_obs.size() * E, 0.0);
    if (which == 1) {  // every item: the source facet's Gauss rule at its point
        std::vector<double> qx, qw;
        gauss_facet(dim, src_far_order, qx, qw);
        for (size_t i = 0; i < tp.i_obs.size(); i++) {
            const Facet& f = fac[tp.i_fac[i]];
            const FacetInfo fi = facet_info(f, dim);
            for (size_t q = 0; q < qw.size(); q++) {
                double bas[3], y[3] = {0, 0, 0};
                if (dim == 2) {
                    bas[0] = 0.5 - 0.5 * qx[2 * q];
                    bas[1] = 0.5 + 0.5 * qx[2 * q];
                    for (int d = 0; d < 2; d++) y[d] = bas[0] * f.c[0].x[d] + bas[1] * f.c[1].x[d];
                } else {
                    bas[0] = 1 - qx[2 * q] - qx[2 * q + 1];
                    bas[1] = qx[2 * q];
                    bas[2] = qx[2 * q + 1];
                    for (int d = 0; d < 3; d++)
                        y[d] = bas[0] * f.c[0].x[d] + bas[1] * f.c[1].x[d] + bas[2] * f.c[2].x[d];
                }
                double K[9];
                oracle_kernel(kernel, mu, nu, &tp.iloc[3 * i], y, pts.normal[tp.i_obs[i]].x, fi.normal.x, K);
                for (int b = 0; b < dim; b++)
                    for (int k = 0; k < R * R; k++)
                        ivals[i * E + b * R * R + k] += bas[b] * (K[k] * fi.jacobian) * qw[q];
            }
        }
    }
    std::vector<double> vals;
    std::vector<long> cols, row_ptr;
    assemble_csr(tp, ivals, (long)pts.loc.size(), nf, dim, R, n_steps, which == 1, vals, cols, row_ptr);
    printf("%ld %ld %zu\n", (long)(row_ptr.size() - 1), R * nf * dim, vals.size());
    for (long r : row_ptr) printf("%ld ", r);
    printf("\n");
    for (long c : cols) printf("%ld ", c);
    printf("\n");
    for (double x : vals) printf("%.17g ", x);
    printf("\n");
    return 0;
}
