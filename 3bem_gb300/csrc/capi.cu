// extern "C" entry points (include/tbem_gpu.h).  Every call catches the
// internal exceptions and turns them into a status code plus a thread-local
// message; nothing aborts.
#include <algorithm>
#include <cstring>
#include <string>

#include "plan.h"

#include "handle.h"

namespace {
thread_local std::string g_last_error;

int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

}  // namespace

namespace tbem {
void set_last_error(const std::string& msg) { g_last_error = msg; }

int api_status()
{
    try {
        throw;
    } catch (const Error& e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(TBEM_ERR_ALLOC, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(TBEM_ERR_ARG, e.what());
    } catch (...) {
        return fail(TBEM_ERR_ARG, "unknown error");
    }
}
}  // namespace tbem

namespace {
template <typename F>
int guarded(F&& f)
{
    try {
        g_last_error.clear();
        f();
        return TBEM_OK;
    } catch (...) {
        return tbem::api_status();
    }
}
}  // namespace

extern "C" {

const char* tbem_last_error(void) { return g_last_error.c_str(); }

void tbem_default_options(TbemGpuOptions* opt)
{
    if (!opt) return;
    std::memset(opt, 0, sizeof(*opt));
    opt->precision = TBEM_PRECISION_FP64;
    opt->device = 0;
    opt->svd_threshold = 1e-10;
    opt->m2l_rank_tol = 1e-7;
}

int tbem_fmm_create(int kernel, const double* kernel_params, const double* obs_locs,
                    const double* obs_normals, long n_obs, const double* src_locs,
                    const double* src_normals, const double* src_weights, long n_src,
                    const TbemFmmConfig* config, const TbemGpuOptions* options, TbemFmm** out)
{
    if (!out || !config) return fail(TBEM_ERR_ARG, "null config or output handle");
    *out = nullptr;
    TbemGpuOptions opt;
    tbem_default_options(&opt);
    if (options) opt = *options;
    TbemFmm* h = nullptr;
    int rc = guarded([&] {
        h = new TbemFmm();
        h->plan.build(kernel, kernel_params, obs_locs, obs_normals, n_obs, src_locs, src_normals,
                      src_weights, n_src, *config, opt);
    });
    if (rc != TBEM_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return TBEM_OK;
}

int tbem_fmm_batch_create(int kernel, const double* kernel_params, int n_meshes,
                          const long* mesh_offsets, const double* locs, const double* normals,
                          const double* weights, const TbemFmmConfig* config,
                          const TbemGpuOptions* options, TbemFmm** out)
{
    if (!out || !config) return fail(TBEM_ERR_ARG, "null config or output handle");
    *out = nullptr;
    TbemGpuOptions opt;
    tbem_default_options(&opt);
    if (options) opt = *options;
    TbemFmm* h = nullptr;
    int rc = guarded([&] {
        h = new TbemFmm();
        h->plan.build_batch(kernel, kernel_params, n_meshes, mesh_offsets, locs, normals, weights,
                            *config, opt);
    });
    if (rc != TBEM_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return TBEM_OK;
}

long tbem_fmm_n_meshes(const TbemFmm* h)
{
    if (!h) return fail(TBEM_ERR_ARG, "null handle");
    return h->plan.batch_off.empty() ? 1 : (long)h->plan.batch_off.size() - 1;
}

int tbem_fmm_apply(TbemFmm* h, const double* x, double* y, int n_rhs, void* stream)
{
    if (!h || !y || (!x && tbem_fmm_n_cols(h) > 0)) return fail(TBEM_ERR_ARG, "null argument");
    return guarded([&] { h->plan.apply(x, y, n_rhs, (cudaStream_t)stream, false); });
}

int tbem_fmm_apply_adjoint(TbemFmm* h, const double* z, double* w, int n_rhs, void* stream)
{
    if (!h || !w || (!z && tbem_fmm_n_rows(h) > 0)) return fail(TBEM_ERR_ARG, "null argument");
    return guarded([&] { h->plan.apply(z, w, n_rhs, (cudaStream_t)stream, true); });
}

int tbem_fmm_source_gradients(TbemFmm* h, const double* x, const double* r, double* g_src_locs,
                              double* g_src_normals, double* g_src_weights, void* stream)
{
    if (!h || (tbem_fmm_n_cols(h) > 0 && (!x || (!r && tbem_fmm_n_rows(h) > 0))))
        return fail(TBEM_ERR_ARG, "null argument");
    return guarded([&] {
        h->plan.source_gradients(x, r, g_src_locs, g_src_normals, g_src_weights, (cudaStream_t)stream);
    });
}

int tbem_fmm_observation_gradients(TbemFmm* h, const double* x, const double* r, double* g_obs_locs,
                                   double* g_obs_normals, void* stream)
{
    if (!h || (tbem_fmm_n_rows(h) > 0 && (!r || (!x && tbem_fmm_n_cols(h) > 0))))
        return fail(TBEM_ERR_ARG, "null argument");
    return guarded([&] {
        h->plan.observation_gradients(x, r, g_obs_locs, g_obs_normals, (cudaStream_t)stream);
    });
}

long tbem_fmm_n_rows(const TbemFmm* h) { return h ? h->plan.R * h->plan.n_obs : TBEM_ERR_ARG; }
long tbem_fmm_n_cols(const TbemFmm* h) { return h ? h->plan.R * h->plan.n_src : TBEM_ERR_ARG; }

int tbem_fmm_clone(const TbemFmm* h, TbemFmm** out)
{
    if (!h || !out) return fail(TBEM_ERR_ARG, "null argument");
    *out = nullptr;
    const tbem::Plan& p = h->plan;
    TbemFmm* c = nullptr;
    const int rc = guarded([&] {
        double params[2] = {p.mu, p.nu};
        // the plan keeps [n][3] points; the create call takes [n][sdim]
        auto narrow = [&](const std::vector<double>& v) {
            std::vector<double> o(v.size() / 3 * p.sdim);
            for (size_t i = 0; i < v.size() / 3; i++)
                for (int d = 0; d < p.sdim; d++) o[p.sdim * i + d] = v[3 * i + d];
            return o;
        };
        const std::vector<double> ol = narrow(p.h_obs_locs), on = narrow(p.h_obs_normals),
                                  sl = narrow(p.h_src_locs), sn = narrow(p.h_src_normals);
        const int created =
            p.batch_off.empty()
                ? tbem_fmm_create(p.kid, params, ol.data(), on.data(), p.n_obs, sl.data(), sn.data(),
                                  p.h_src_weights.data(), p.n_src, &p.cfg, &p.opt, &c)
                : tbem_fmm_batch_create(p.kid, params, (int)p.batch_off.size() - 1,
                                        p.batch_off.data(), sl.data(), sn.data(),
                                        p.h_src_weights.data(), &p.cfg, &p.opt, &c);
        if (created != TBEM_OK) throw tbem::Error(created, g_last_error);
        if (!p.f.mixed && !p.opt.host_only) {
            // carry over installed check-to-equivalent operators (a host-only
            // operator has none)
            std::vector<double> buf((size_t)p.n * p.n);
            for (int w = 0; w < 2; w++) {
                long nl = (long)(w == 0 ? p.f.c2e_up_off.size() : p.f.c2e_dn_off.size());
                for (long l = 0; l < nl; l++) {
                    p.get_c2e(w, l, buf.data());
                    c->plan.set_c2e(w, l, buf.data());
                }
            }
        }
    });
    if (rc != TBEM_OK) {
        delete c;
        return rc;
    }
    *out = c;
    return TBEM_OK;
}

void tbem_fmm_destroy(TbemFmm* h) { delete h; }

long tbem_fmm_tree_cells(const TbemFmm* h, int which, long* level, long* index, double* center,
                         double* half_width, long* n_points, long* n_children)
{
    if (!h || (which != 0 && which != 1)) return fail(TBEM_ERR_ARG, "bad handle or tree");
    const tbem::Tree& t = which == 0 ? *h->plan.stree : h->plan.otree;
    for (size_t k = 0; k < t.preorder.size(); k++) {
        const tbem::Cell& c = t.cells[t.preorder[k]];
        if (level) level[k] = c.level;
        if (index) index[k] = c.ref_index;
        if (center) for (int d = 0; d < 3; d++) center[3 * k + d] = c.center[d];
        if (half_width) for (int d = 0; d < 3; d++) half_width[3 * k + d] = c.hw[d];
        if (n_points) n_points[k] = c.n_points();
        if (n_children) n_children[k] = c.n_children;
    }
    return (long)t.preorder.size();
}

long tbem_fmm_tree_indices(const TbemFmm* h, int which, long* out)
{
    if (!h || (which != 0 && which != 1)) return fail(TBEM_ERR_ARG, "bad handle or tree");
    const tbem::Tree& t = which == 0 ? *h->plan.stree : h->plan.otree;
    long k = 0;
    const int rc = guarded([&] {
        std::vector<long> tmp;
        for (int f : t.preorder) {
            const tbem::Cell& c = t.cells[f];
            // the reference lists a cell's points in ascending original order
            tmp.assign(t.perm.begin() + c.pt_begin, t.perm.begin() + c.pt_end);
            std::sort(tmp.begin(), tmp.end());
            for (long v : tmp) {
                if (out) out[k] = v;
                k++;
            }
        }
    });
    return rc != TBEM_OK ? rc : k;
}

long tbem_fmm_list(const TbemFmm* h, int kind, long* obs_index, long* src_index)
{
    if (!h || kind < 0 || kind > 7) return fail(TBEM_ERR_ARG, "bad handle or list kind");
    const tbem::Plan& p = h->plan;
    const tbem::Tree& O = p.otree;
    const tbem::Tree& S = *p.stree;
    auto cells = [&](const std::vector<int>& v, const tbem::Tree& t) {
        for (size_t i = 0; i < v.size(); i++) {
            if (obs_index) obs_index[i] = t.cells[v[i]].ref_index;
            if (src_index) src_index[i] = -1;
        }
        return (long)v.size();
    };
    auto pairs = [&](const std::vector<tbem::CellPair>& v) {
        for (size_t i = 0; i < v.size(); i++) {
            if (obs_index) obs_index[i] = O.cells[v[i].obs].ref_index;
            if (src_index) src_index[i] = S.cells[v[i].src].ref_index;
        }
        return (long)v.size();
    };
    switch (kind) {
    case 0: return cells(p.L.p2m, S);
    case 1: return cells(p.L.m2m, S);
    case 2: return pairs(p.L.p2p);
    case 3: return pairs(p.L.m2p);
    case 4: return pairs(p.L.p2l);
    case 5: return pairs(p.L.m2l);
    case 6: return cells(p.L.l2l, O);
    default: return cells(p.L.l2p, O);
    }
}

long tbem_fmm_n_surface(const TbemFmm* h) { return h ? h->plan.ns : TBEM_ERR_ARG; }

long tbem_fmm_n_c2e_levels(const TbemFmm* h, int which)
{
    if (!h || (which != 0 && which != 1)) return fail(TBEM_ERR_ARG, "bad handle");
    return (long)(which == 0 ? h->plan.f.c2e_up_off.size() : h->plan.f.c2e_dn_off.size());
}

int tbem_fmm_get_c2e(const TbemFmm* h, int which, long level, double* out)
{
    if (!h || !out) return fail(TBEM_ERR_ARG, "null argument");
    return guarded([&] { h->plan.get_c2e(which, level, out); });
}

int tbem_fmm_set_c2e(TbemFmm* h, int which, long level, const double* op)
{
    if (!h || !op) return fail(TBEM_ERR_ARG, "null argument");
    return guarded([&] { h->plan.set_c2e(which, level, op); });
}

long tbem_fmm_p2p_block(const TbemFmm* h) { return h ? h->plan.p2p_tpt : TBEM_ERR_ARG; }

long tbem_fmm_tc_tile(const TbemFmm* h)
{
    if (!h) return TBEM_ERR_ARG;
    if (h->plan.f.use_tc_c) return h->plan.f.m2l_c.tc_bn;
    return h->plan.f.use_tc ? h->plan.f.m2l.tc_bn : 0;
}

int tbem_fmm_m2l_ranks(const TbemFmm* h, long* r_in, long* r_out)
{
    if (!h) return fail(TBEM_ERR_ARG, "null handle");
    const bool c = h->plan.f.m2l_compressed;
    if (r_in) *r_in = c ? h->plan.f.r_in : 0;
    if (r_out) *r_out = c ? h->plan.f.r_out : 0;
    return TBEM_OK;
}

int tbem_fmm_graph_create(TbemFmm* const* ops, int n_ops, const double* const* x, double* const* y,
                          int n_rhs, int adjoint, TbemGraph** out)
{
    if (!out) return fail(TBEM_ERR_ARG, "null output handle");
    *out = nullptr;
    TbemGraph* g = nullptr;
    int rc = guarded([&] {
        g = tbem::graph_new();
        tbem::graph_build(*g, ops, n_ops, x, y, n_rhs, adjoint != 0);
    });
    if (rc != TBEM_OK) {
        tbem::graph_delete(g);
        return rc;
    }
    *out = g;
    return TBEM_OK;
}

int tbem_fmm_graph_launch(TbemGraph* g, void* stream)
{
    if (!g) return fail(TBEM_ERR_ARG, "null graph");
    return guarded([&] { tbem::graph_launch(*g, (cudaStream_t)stream); });
}

void tbem_fmm_graph_destroy(TbemGraph* g) { tbem::graph_delete(g); }

long tbem_fmm_last_launches(const TbemFmm* h) { return h ? h->plan.launches : TBEM_ERR_ARG; }

int tbem_fmm_sync(TbemFmm* h, void* stream)
{
    if (!h) return fail(TBEM_ERR_ARG, "null handle");
    return guarded([&] { h->plan.sync((cudaStream_t)stream); });
}

int tbem_fmm_set_wait_cycles(TbemFmm* h, long long cycles)
{
    if (!h) return fail(TBEM_ERR_ARG, "null handle");
    if (cycles < 0) return fail(TBEM_ERR_ARG, "negative wait budget");
    h->plan.f.tc.wait_cycles = cycles;
    h->plan.f.tc_c.wait_cycles = cycles;
    return TBEM_OK;
}

int tbem_fmm_set_timing(TbemFmm* h, int enabled)
{
    if (!h) return fail(TBEM_ERR_ARG, "null handle");
    h->plan.timing = enabled != 0;
    return TBEM_OK;
}

int tbem_fmm_phase_times(const TbemFmm* h, const char** names, double* ms, int cap)
{
    if (!h) return fail(TBEM_ERR_ARG, "null handle");
    int rc = guarded([&] { const_cast<TbemFmm*>(h)->plan.read_phases(); });
    if (rc != TBEM_OK) return rc;
    const auto& v = h->plan.phase_ms;
    int k = 0;
    for (size_t i = 0; i < v.size(); i++, k++) {
        if (k >= cap) continue;
        if (names) names[k] = v[i].first.c_str();
        if (ms) ms[k] = v[i].second;
    }
    return k;
}

int tbem_fmm_setup_times(const TbemFmm* h, const char** names, double* seconds, int cap)
{
    if (!h) return fail(TBEM_ERR_ARG, "null handle");
    const auto& v = h->plan.setup_s;
    int k = 0;
    for (size_t i = 0; i < v.size(); i++, k++) {
        if (k >= cap) continue;
        if (names) names[k] = v[i].first.c_str();
        if (seconds) seconds[k] = v[i].second;
    }
    return k;
}

}  // extern "C"
