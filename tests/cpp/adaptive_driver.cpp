// Test driver: the product's level-by-level adaptive Gauss-Lobatto engine
// (3bem_gb300/csrc/nearfield_adaptive.cpp) with the oracle's CPU kernels as
// the point evaluator, so that tests/test_nearfield_host.py can compare its
// facet integrals with the reference's recursive integrator on the CPU.  The
// product evaluates the same points on the GPU.
//
// argv[1] (optional): terms per breadth-first batch.
// stdin: kernel mu nu tol dim, then per term: obs[3] normal[3] facet[dim][3]
// (until EOF); stdout: dim * R * R values per term.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "nearfield.h"

extern "C" int oracle_kernel(int kernel, double mu, double nu, const double* obs, const double* src,
                             const double* nobs, const double* nsrc, double* out);

using namespace tbem::nf;

int main(int argc, char** argv)
{
    const long slice = argc > 1 ? atol(argv[1]) : (1L << 18);
    int kernel, dim;
    double mu, nu, tol;
    if (scanf("%d %lf %lf %lf %d", &kernel, &mu, &nu, &tol, &dim) != 5) return 1;
    std::vector<V3> loc, nrm;
    std::vector<Facet> fac;
    while (true) {
        V3 p{}, n{};
        Facet f{};
        if (scanf("%lf %lf %lf %lf %lf %lf", &p.x[0], &p.x[1], &p.x[2], &n.x[0], &n.x[1], &n.x[2]) != 6) break;
        for (int v = 0; v < dim; v++)
            for (int d = 0; d < 3; d++)
                if (scanf("%lf", &f.c[v].x[d]) != 1) return 1;
        loc.push_back(p);
        nrm.push_back(n);
        fac.push_back(f);
    }
    double probe[9];
    const double z[3] = {0, 0, 0}, one[3] = {1, 0, 0};
    const int RR = oracle_kernel(kernel, mu, nu, z, one, one, one, probe);
    const int E = dim * RR;
    const int R = RR == 9 ? 3 : RR == 4 ? 2 : 1;
    InfluenceEval eval = [&](const std::vector<long>& item, const std::vector<double>& x0,
                             const std::vector<double>& x1, std::vector<double>& out) {
        out.assign(item.size() * E, 0.0);
        for (size_t k = 0; k < item.size(); k++) {
            const Facet& f = fac[item[k]];
            const FacetInfo fi = facet_info(f, dim);
            double bas[3], y[3] = {0, 0, 0};
            if (dim == 2) {
                bas[0] = 0.5 - 0.5 * x0[k];
                bas[1] = 0.5 + 0.5 * x0[k];
                for (int d = 0; d < 2; d++) y[d] = bas[0] * f.c[0].x[d] + bas[1] * f.c[1].x[d];
            } else {
                bas[0] = 1 - x0[k] - x1[k];
                bas[1] = x0[k];
                bas[2] = x1[k];
                for (int d = 0; d < 3; d++)
                    y[d] = bas[0] * f.c[0].x[d] + bas[1] * f.c[1].x[d] + bas[2] * f.c[2].x[d];
            }
            double K[9];
            oracle_kernel(kernel, mu, nu, loc[item[k]].x, y, nrm[item[k]].x, fi.normal.x, K);
            for (int b = 0; b < dim; b++)
                for (int q = 0; q < R * R; q++) out[k * E + b * R * R + q] = bas[b] * (K[q] * fi.jacobian);
        }
    };
    const std::vector<double> v = adaptive_facet_integrals(dim, E, (long)loc.size(), tol, eval, slice);
    for (size_t t = 0; t < loc.size(); t++) {
        for (int e = 0; e < E; e++) printf("%.17g ", v[t * E + e]);
        printf("\n");
    }
    return 0;
}
