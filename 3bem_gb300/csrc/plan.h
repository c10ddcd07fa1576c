// FMM plan: everything built once per geometry (the reference's FMMOperator
// constructor, cpp/fmm.cpp:72-101) and the apply sequences.
#pragma once
#include <cublas_v2.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <map>
#include <memory>
#include <tuple>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tbem_gpu.h"
#include "eval_launch.h"
#include "gemm.cuh"
#include "kernels.cuh"
#include "tree.h"

namespace tbem {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Records the message returned by tbem_last_error() on the calling thread.
void set_last_error(const std::string& msg);

// Inside a catch block of an extern "C" entry point: records the exception
// being handled as the calling thread's last error and returns its status
// (tbem::Error: its code; std::bad_alloc: TBEM_ERR_ALLOC; any other
// exception: TBEM_ERR_ARG), so that no C++ exception crosses the C ABI.
int api_status();

void check_cuda(cudaError_t e, const char* what, const char* file, int line);
// empties the process's cache of factored pseudo-inverses and M2L eigenbases
void clear_setup_cache();
void check_cublas(cublasStatus_t e, const char* what, const char* file, int line);
void check_cusolver(cusolverStatus_t e, const char* what, const char* file, int line);
#define TBEM_CK(x) ::tbem::check_cuda((x), #x, __FILE__, __LINE__)
#define TBEM_CKB(x) ::tbem::check_cublas((x), #x, __FILE__, __LINE__)
#define TBEM_CKS(x) ::tbem::check_cusolver((x), #x, __FILE__, __LINE__)

// Makes dev current for a scope and gives the caller's device back after it,
// so that operators on different GPUs can be used from one thread.
struct DeviceGuard {
    int prev = -1;
    bool changed = false;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            cudaGetLastError();
            prev = -1;
        }
        if (prev != dev) {
            check_cuda(cudaSetDevice(dev), "cudaSetDevice", __FILE__, __LINE__);
            changed = true;
        }
    }
    ~DeviceGuard()
    {
        if (changed && prev >= 0) cudaSetDevice(prev);
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
};

// Owning device buffer.
template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DBuf& operator=(DBuf&& o) noexcept
    {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count)
    {
        if (count == n && p) return;
        release();
        if (count == 0) return;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            throw Error(TBEM_ERR_ALLOC, "cudaMalloc of " + std::to_string(count * sizeof(T)) +
                                            " bytes failed: " + cudaGetErrorString(e));
        }
        n = count;
    }
    void ensure(size_t count)
    {
        if (count > n) alloc(count);
    }
    // Setup-time copies.  The plans compute on non-blocking streams, which a
    // plain cudaMemcpy (legacy default stream) does not order against: an
    // upload waits for its DMA to land, a download for all device work.
    void upload(const std::vector<T>& v) { upload(v.data(), v.size()); }
    void upload(const T* src, size_t count)
    {
        alloc(count);
        if (count) {
            TBEM_CK(cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice));
            TBEM_CK(cudaStreamSynchronize(cudaStreamLegacy));
        }
    }
    // The same into the first v.size() elements, growing the buffer only when
    // it is too small: repeated uploads of varying sizes keep one allocation.
    void upload_grow(const std::vector<T>& v)
    {
        ensure(v.size());
        if (!v.empty()) {
            TBEM_CK(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
            TBEM_CK(cudaStreamSynchronize(cudaStreamLegacy));
        }
    }
    std::vector<T> download() const
    {
        std::vector<T> v(n);
        if (n) {
            TBEM_CK(cudaDeviceSynchronize());
            TBEM_CK(cudaMemcpy(v.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost));
        }
        return v;
    }
};

// A timing event destroyed on every exit path (the autotuners time
// candidates between two of these).
struct ScopedEvent {
    cudaEvent_t e = nullptr;
    ScopedEvent() { TBEM_CK(cudaEventCreate(&e)); }
    ScopedEvent(const ScopedEvent&) = delete;
    ScopedEvent& operator=(const ScopedEvent&) = delete;
    ~ScopedEvent()
    {
        if (e) cudaEventDestroy(e);
    }
};

// A set of obs-owner evaluation tasks (eval.cuh).
struct TaskSet {
    std::vector<long> tgt;
    std::vector<int> tgt_count;
    std::vector<double> origin;
    std::vector<int> src_ptr{0};
    std::vector<long> blk;
    std::vector<int> blk_count, blk_prefix;
    std::vector<int> blk_near;  // per block: its cell touches the target leaf (point-to-point sets)
    std::vector<int> item_task, item_start;
    DBuf<long> d_tgt, d_blk;
    DBuf<int> d_tgt_count, d_src_ptr, d_blk_count, d_blk_prefix, d_item_task, d_item_start, d_blk_near;
    DBuf<double> d_origin;
    long n_pairs = 0;  // sum over tasks of targets x sources (work estimate)
    int tpt = 4;       // threads per target the items were cut for

    int n_tasks() const { return (int)tgt.size(); }
    int n_items() const { return (int)item_task.size(); }
    // near: one flag per entry of srcs (empty: no flags)
    void add(long target, int count, const double* org, const std::vector<std::pair<long, int>>& srcs,
             int targets_per_cta, const std::vector<int>& near = {});
    void upload();
    template <typename T>
    void fill(EvalArgs<T>& a) const
    {
        a.item_task = d_item_task.p;
        a.item_start = d_item_start.p;
        a.task_tgt = d_tgt.p;
        a.task_tgt_count = d_tgt_count.p;
        a.task_origin = d_origin.p;
        a.task_src_ptr = d_src_ptr.p;
        a.src_blk = d_blk.p;
        a.src_blk_count = d_blk_count.p;
        a.src_blk_prefix = d_blk_prefix.p;
        a.src_blk_near = d_blk_near.p;
    }
};

// Three-term bf16 planes of the precision form's FP32 operators, padded for
// the tensor-core GEMM (tc_gemm.cu), plus the split of the current B operand.
struct TcPlanes {
    int m = 0, k = 0, m_pad = 0, k_pad = 0;  // operators m x k (row-major)
    DBuf<__nv_bfloat16> a[3], b[3];
    DBuf<int> err;  // set by a tensor-core GEMM whose bounded wait gave up
    long long wait_cycles = 0;  // budget of the GEMM's bounded waits (0: the default)
    void build(const float* ops32, long n_ops, int m, int k, cudaStream_t s);
    void split_b(const float* cells, long rows, cudaStream_t s);
    // split only rows [row0, row0 + rows) of a [rows_total][k] buffer into
    // the same rows of the planes (capacity for rows_total rows)
    void split_b_rows(const float* cells, long row0, long rows, long rows_total, cudaStream_t s);
};

// A set of GEMM groups (gemm.cuh) sharing B and D buffers.
struct GemmSet {
    std::vector<long> A_off;  // operator offsets (elements) into an operator pool
    std::vector<long> pair0;
    std::vector<int> npairs;
    std::vector<int> in_cell, out_cell;
    DBuf<long> d_pair0;
    DBuf<int> d_npairs, d_in, d_out;
    DBuf<const void*> d_A;  // resolved pointers
    std::map<int, std::pair<DBuf<int>, DBuf<int>>> tiles;  // per nrhs
    // conflict-free waves for GEMM_WAVES (built on first use)
    std::vector<int> wave_of;
    int n_waves = 0;
    std::map<int, std::vector<int>> wave_tile_start;  // per nrhs: first tile of every wave
    void build_waves();
    long total_pairs() const { return (long)in_cell.size(); }
    bool empty() const { return in_cell.empty(); }
    void add_group(long a_off, const std::vector<std::pair<int, int>>& pairs);
    void upload(const void* pool, size_t elem_size);
    template <typename T>
    void run(const T* B, T* D, int n, int nrhs, int trans, int mode, cudaStream_t s,
             long* launches = nullptr)
    {
        run_rect<T>(B, D, n, n, n, nrhs, trans, mode, s, launches);
    }
    // op(A) is m x k; A is stored row-major with rows of length lda
    template <typename T>
    void run_rect(const T* B, T* D, int m, int k, int lda, int nrhs, int trans, int mode,
                  cudaStream_t s, long* launches = nullptr, bool tables_only = false);
    // tensor-core path (B taken from P's split planes; D columns of P.m rows);
    // nn = elements per operator in the pool the groups' offsets refer to
    struct TcTiles {
        DBuf<int4> t;  // per column tile: operator, group's first pair, first column, group columns
        DBuf<int> brow, drow;  // per column tile and column (when small): B row / D column, -1 past the end
        int n = 0;
    };
    std::map<int, TcTiles> tc_tiles;  // per (nrhs, N tile)
    int tc_bn = 128;  // N tile of the tensor-core path (128 or 64; autotuned)
    int tc_bk = 64;   // K chunk (64, or 32 with N = 128; autotuned)
    void run_tc(const TcPlanes& P, float* D, int nrhs, int atomic, long nn, cudaStream_t s,
                long* launches);
};

// Deterministic accumulation of a GEMM set whose groups add into the same
// outputs (the plain form's M2L: every observation cell receives one product
// per source of its interaction list).  Every pair's product is stored in a
// slot of its own -- one GEMM launch over all groups, [slot][rhs][m] -- and
// each output column then sums its slots in pair order: a fixed summation
// order with no atomics and two launches per chunk.  The pairs run in chunks
// of at most `cap` slots, which bounds the slot buffer.
struct SlotPlan {
    struct Chunk {
        GemmSet gemm;             // the chunk's groups, out_cell = local slot
        DBuf<int> tgt, ptr, idx;  // output cells with slots, CSR of their local slots
        int n_tgt = 0;
    };
    std::vector<Chunk> chunks;
    long max_slots = 0;
    bool empty() const { return chunks.empty(); }
    void build(const GemmSet& G, long cap, const void* pool, size_t esz);
    // D[out][rhs][:] += sum over the pairs of op(A_g) B[in][rhs][:]
    void run(const double* B, double* D, int m, int nrhs, int trans, double* slots, cudaStream_t s,
             long* launches);
};

struct DTree {
    DBuf<double> center, rad, xyz, w;
    DBuf<double> nrm64;
    DBuf<float> nrm32;
    DBuf<long> perm;
};

// Operators and task sets of one precision form.
struct Form {
    bool mixed = false;
    // kernels of the form: translations / check-to-equivalent systems use
    // g_kid, real sources enter the check surfaces through ks_kid and the
    // equivalent sources reach the targets through kt_kid (all equal to the
    // operator's kernel in the plain form)
    int g_kid = 0, ks_kid = 0, kt_kid = 0;
    double r_ue = 0, r_uc = 0, r_dc = 0, r_de = 0;
    std::vector<long> c2e_up_off, c2e_dn_off;  // offsets into c2e pool (FP64, n x n)
    DBuf<double> c2e;
    DBuf<double> ops64;                         // plain: Mop, Lop, T_k
    DBuf<float> ops32;                          // mixed: combined M2M', L2L', U_k
    std::vector<GemmSet> c2e_up, m2m, l2l, c2e_dn;  // per level
    GemmSet m2l;
    // plain form: the M2L products through slots (deterministic, no waves)
    SlotPlan m2l_slots, m2l_t_slots;
    // transposed sets (in/out swapped) for the adjoint apply
    std::vector<GemmSet> c2e_up_t, m2m_t, l2l_t, c2e_dn_t;
    GemmSet m2l_t;
    bool m2l_on_the_fly = false;
    // mixed: tensor-core planes of ops32 (M2L on tcgen05 when use_tc)
    TcPlanes tc;
    bool use_tc = false;
    // compressed form: tensor-core planes of the C_k (m2l_path 5)
    TcPlanes tc_c;
    bool use_tc_c = false;
    bool use_tc_updown = false;
    // mixed, compressed (m2l_path 0 / 4): the far field runs in the SVD bases
    // of the M2L kernel matrices.  Upward states are r_in coefficients
    // u~ = P_l u, downward states r_out coefficients (d ~= V d~).  All
    // operators row-major FP32:
    //   Pb   per source level  P_l (r_in x n): leaf check potentials -> u~
    //   Wl   per source level  2^-l W (n x r_in): u~ -> equivalent densities (M2P)
    //   Vb   V (n x r_out): down-check potentials <-> d~ (P2L)
    //   Cops per M2L class     C_k (r_out x r_in)
    //   Xops per M2M operator  X (r_in x r_in)
    //   Yops per L2L operator  Y (r_out x r_out)
    // and the L2P operators E take d~ directly (E V).
    bool m2l_compressed = false;
    int r_in = 0, r_out = 0;
    DBuf<float> Pb, Wl, Vb, Cops, Xops, Yops;
    // the FP64 compressed form (TBEM_PRECISION_FP64_COMPRESSED): the same
    // operators kept in FP64 and applied on the FP64 pipes
    bool f64 = false;
    DBuf<double> Pb64, Wl64, Vb64, Cops64, Xops64, Yops64, E64;
    DBuf<double> V64;  // V in FP64 (column-major n x r_out) while the L2P operators are built
    GemmSet m2l_c, m2l_c_t, comp_p2m, decomp_m2p, comp_p2l;
    GemmSet decomp_l2p;  // V over the L2P leaves: their down-check potentials (gradients)
    std::vector<GemmSet> m2m_c, m2m_c_t, l2l_c, l2l_c_t;  // per level
    // mixed: per-leaf L2P operators
    DBuf<float> E;
    DBuf<long> E_row0;  // per l2p task
    DBuf<int> E_leaf, E_npts;
    DBuf<long> E_pt0;
    int n_l2p = 0;
    int E_ld = 0;  // padded row stride of E (multiple of 128 floats)
};

struct Plan {
    int kid = 0, R = 1;
    int sdim = 3;  // space dimension of the kernel (2: the reference's FMMOperator<2,R,C>)
    double mu = 1.0, nu = 0.25;
    KParams kp{};
    TbemFmmConfig cfg{};
    TbemGpuOptions opt{};
    long n_obs = 0, n_src = 0;
    int ns = 0, n = 0;
    bool same_tree = false;
    // precision forms with different observation and source points: both
    // trees cut from one bounding cube (integer M2L offsets between them)
    bool common_cube = false;
    Tree otree, stree_own;
    const Tree* stree = nullptr;
    TaskLists L;
    std::vector<double> unit;
    DBuf<double> d_unit;
    DTree dobs, dsrc_own;
    DTree* dsrc = nullptr;
    Form f;
    // evaluation task sets (forward); adjoint sets swap roles
    TaskSet p2m, p2p, m2p, p2l, l2p, m2l_fly;
    // point-to-point variants for 2 and 8 threads per target (autotuned)
    TaskSet p2p_tpt2, p2p_tpt8;
    int p2p_tpt = 4;
    // points-to-check-surface variants for 1 and 2 threads per target (autotuned)
    TaskSet p2m_tpt1, p2m_tpt2;
    int p2m_tpt = 4;
    void autotune_p2m();
    const TaskSet& p2m_set() const { return p2m_tpt == 1 ? p2m_tpt1 : p2m_tpt == 2 ? p2m_tpt2 : p2m; }
    void autotune_p2p();
    void autotune_tc();  // N tile (128 / 64) of the tensor-core translations
    const TaskSet& p2p_set() const { return p2p_tpt == 2 ? p2p_tpt2 : p2p_tpt == 8 ? p2p_tpt8 : p2p; }
    TaskSet p2m_t, p2p_t, m2p_t, p2l_t, l2p_t, m2l_fly_t;
    // work buffers
    int cap_rhs = 0;
    DBuf<double> io_x, io_y;            // device staging of caller data (original order)
    double* xin = nullptr;              // the current chunk of right-hand sides in io_x
    double* yout = nullptr;             // and its outputs in io_y
    int rhs_chunk(int nrhs) const;
    DBuf<double> s64, y64;              // strengths / outputs in tree order
    DBuf<float> s32;
    DBuf<double> cu64, qu64, cd64, qd64;  // cell buffers [cell][rhs][n]
    DBuf<double> slots64;                 // plain form: M2L product slots [slot][rhs][n]
    DBuf<float> cu32, cd32;
    DBuf<float> cuc32, cdc32;  // compressed M2L coefficients [cell][rhs][r_in | r_out]
    DBuf<double> cuc64, cdc64;  // the same in the FP64 compressed form
    cudaStream_t stream = nullptr;
    // second stream for the near field, which runs beside the far-field
    // passes of the compressed form (forked after the gather, joined before
    // the passes that add into the outputs)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cublasHandle_t cublas = nullptr;
    cusolverDnHandle_t solver = nullptr;
    // timeout flags of the bounded device waits (the tensor-core GEMMs)
    // copied to pinned memory after every apply; an apply with device
    // outputs reports a flag raised by the previous one
    static constexpr int N_ERR_FLAGS = 4;
    int* h_err = nullptr;
    void check_tc_flags(bool wait_device, cudaStream_t s);
    std::vector<const int*> device_flags() const;
    bool flags_raised() const;
    // waits for the plan's work (and stream s) and throws TBEM_ERR_TIMEOUT
    // if a tensor-core pass of any earlier apply gave up
    void sync(cudaStream_t s);
    bool timing = false;
    long launches = 0;  // kernel launches of the last apply
    // phase timing: events recorded on the apply's stream (no synchronization);
    // read_phases() turns the marks of the applies since the last read into
    // mean milliseconds per apply
    std::vector<std::pair<std::string, cudaEvent_t>> marks;
    std::vector<cudaEvent_t> event_pool;
    std::vector<std::pair<std::string, double>> phase_ms;
    void read_phases();
    // construction phases: wall seconds of each, the device synchronized at
    // every mark (host work, uploads, factorisations, operator tables,
    // autotuning)
    std::vector<std::pair<std::string, double>> setup_s;
    double setup_t = 0;  // time of the last mark (steady clock seconds)
    void setup_start();
    void setup_mark(const char* name);
    // kept for clone()
    std::vector<double> h_obs_locs, h_obs_normals, h_src_locs, h_src_normals, h_src_weights;
    // batched form (build_batch): mesh m owns points [batch_off[m],
    // batch_off[m + 1]); its centre and half width map it into [-1, 1]^3.
    // Empty for a single-mesh operator.
    std::vector<long> batch_off;
    std::vector<double> batch_center, batch_scale;

    ~Plan();
    void build(int kernel, const double* params, const double* obs_locs, const double* obs_normals,
               long n_obs, const double* src_locs, const double* src_normals,
               const double* src_weights, long n_src, const TbemFmmConfig& cfg,
               const TbemGpuOptions& opt);
    void build_batch(int kernel, const double* params, int n_meshes, const long* offsets,
                     const double* locs, const double* normals, const double* weights,
                     const TbemFmmConfig& cfg, const TbemGpuOptions& opt);
    void create_streams();
    void finish_build(const double* o_locs, const double* o_nrm, const double* s_locs,
                      const double* s_nrm, const double* s_w);
    void apply(const double* x, double* y, int nrhs, cudaStream_t s, bool adjoint);
    // Derivatives of L = r^T A x with respect to the source points'
    // positions, normals and weights (device arrays [n_src][3], [n_src][3],
    // [n_src] in the caller's order; any may be null) through the transposed
    // passes of the compressed forms (grad.cu).
    void source_gradients(const double* x, const double* r, double* g_y, double* g_n, double* g_w,
                          cudaStream_t s);
    // The same for the observation points' positions and normals
    // ([n_obs][3] each): one forward apply, then its passes that reach
    // observation points with the kernel's derivatives (grad.cu).
    void observation_gradients(const double* x, const double* r, double* g_x, double* g_n,
                               cudaStream_t s);
    DBuf<double> grad_buf;  // source_gradients' work arrays
    void set_c2e(int which, long level, const double* op);
    void get_c2e(int which, long level, double* out) const;

    void upload_tree(const Tree& t, const double* locs, const double* normals,
                     const double* weights, DTree& d);
    void build_tasks();
    void build_form();
    void build_c2e(Form& F);
    void build_plain_ops(Form& F);
    void build_mixed_ops(Form& F);
    struct CompressionInput {
        const double* T0;                  // root-scaled M2L kernel matrices (compact)
        long n_m2l;
        const std::vector<long>* m2l_index;  // job -> compact M2L index
        const double* KM;                  // M2M kernel matrices (compact)
        const std::vector<int>* m2m_lc;    // compact M2M -> child level
        const std::vector<long>* m2m_index;
        const double* YL;                  // combined L2L operators (compact)
        const std::vector<long>* l2l_index;
        const std::vector<long>* m2m_off;
        const std::vector<long>* l2l_off;
        uint64_t t0_key[2];                // two hashes of what the M2L matrices depend on
    };
    void build_compression(Form& F, const CompressionInput& in);
    // T = float: the precision form; T = double: the FP64 compressed form
    template <typename T>
    void forward_compressed(int nrhs, cudaStream_t s);
    template <typename T>
    void adjoint_compressed(int nrhs, cudaStream_t s);
    void build_gemm_sets(Form& F, long op_base_m2m, long op_base_l2l, long op_base_m2l,
                         const std::vector<long>& m2m_off, const std::vector<long>& l2l_off,
                         const std::vector<long>& m2l_off);
    void ensure_rhs(int nrhs);
    void forward(int nrhs, cudaStream_t s);
    void adjoint(int nrhs, cudaStream_t s);
    template <typename T>
    void eval(const TaskSet& ts, int ekid, bool tgt_surf, bool src_surf, const Tree& tt,
              const DTree& dt, double t_rref, const DTree& ds, double s_rref, const T* s_str,
              long s_n, const T* q, double* y, long y_n, T* c, int add, int nrhs, cudaStream_t s,
              bool trans);
    void mark(const char* name, cudaStream_t s);
    template <typename T>
    void launch_l2p(const T* cd, int len, int nrhs, cudaStream_t s);
    size_t l2p_smem_set[2] = {0, 0};  // dynamic shared memory opted in for the many-RHS L2P (FP32, FP64)
    // operator pool layout of the current form
    std::vector<int> m2m_key_level, l2l_key_level;
    std::vector<std::vector<int>> m2l_groups;  // pair indices per M2L key
    std::vector<int> m2l_key_ls;               // source level per key
    std::vector<std::pair<int, int>> m2l_canon;
    std::vector<std::vector<std::pair<int, int>>> m2m_pairs, l2l_pairs;  // per (level*8+oct)
    std::vector<std::pair<int, int>> m2m_canon, l2l_canon;
};

}  // namespace tbem
