// Direct FP64 N-body sum that allocates nothing (tbem_direct_apply_noalloc).
//
// Some callers cannot call cudaMalloc: applications whose device memory is
// owned by another allocator under a fixed budget (a framework's caching pool,
// an embedded solver with pre-reserved memory), real-time loops where an
// allocation's latency or its implicit device synchronisation is not
// acceptable, and plugins that the host program forbids from allocating.
// This entry point serves them: the caller passes device inputs and outputs,
// and the kernel's scratch (the weighted source strengths and the work-item
// descriptors) lives in one file-scope static device array of
// NOALLOC_SCRATCH_BYTES (16 MiB), which every GPU that loads the library keeps
// until the process exits.
//
// The array's host-side name is only a stand-in for the device object, so
// its device address is looked up with cudaGetSymbolAddress on every call,
// with the caller's device current.  Nothing is cached: after a device reset
// (or any teardown of the primary context) the runtime loads the module
// again and the lookup returns the new address.  The first call on a device
// loads the module there, so make it before any stream capture.  All calls
// share the array and it keeps the last call's contents; everything this
// path reads from it is rewritten by the same call before use.  Two calls
// whose work overlaps on the GPU (for example on two streams) race on the
// array.
#include "plan.h"

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(16) << 20;
constexpr size_t NOALLOC_TASK_BYTES = size_t(1) << 20;     // work-item descriptors
constexpr int NOALLOC_CHUNK = 1024;                        // observation points per task
constexpr int NOALLOC_TPB = tbem::EVAL_THREADS / 4;        // targets per CTA (4 threads each)

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array on the current device.
unsigned char* scratch_address()
{
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        throw tbem::Error(TBEM_ERR_CUDA, std::string("cudaGetSymbolAddress of the scratch "
                                                     "array failed: ") + cudaGetErrorString(e));
    }
    return static_cast<unsigned char*>(p);
}

struct TaskLayout {
    size_t item_task, item_start, task_tgt, task_count, task_origin, src_ptr, blk, blk_count,
        blk_prefix, total;
};

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

TaskLayout layout(int n_tasks, int n_items)
{
    TaskLayout L;
    size_t o = 0;
    L.item_task = o; o = align256(o + sizeof(int) * n_items);
    L.item_start = o; o = align256(o + sizeof(int) * n_items);
    L.task_tgt = o; o = align256(o + sizeof(long) * n_tasks);
    L.task_count = o; o = align256(o + sizeof(int) * n_tasks);
    L.task_origin = o; o = align256(o + sizeof(double) * 3 * n_tasks);
    L.src_ptr = o; o = align256(o + sizeof(int) * (n_tasks + 1));
    L.blk = o; o = align256(o + sizeof(long) * n_tasks);
    L.blk_count = o; o = align256(o + sizeof(int) * n_tasks);
    L.blk_prefix = o; o = align256(o + sizeof(int) * n_tasks);
    L.total = o;
    return L;
}

// One task per chunk of observation points, each against all sources.
__global__ void noalloc_fill_tasks(unsigned char* base, TaskLayout L, long n_obs, int n_src,
                                   int n_tasks, int n_items)
{
    int* item_task = reinterpret_cast<int*>(base + L.item_task);
    int* item_start = reinterpret_cast<int*>(base + L.item_start);
    long* task_tgt = reinterpret_cast<long*>(base + L.task_tgt);
    int* task_count = reinterpret_cast<int*>(base + L.task_count);
    double* task_origin = reinterpret_cast<double*>(base + L.task_origin);
    int* src_ptr = reinterpret_cast<int*>(base + L.src_ptr);
    long* blk = reinterpret_cast<long*>(base + L.blk);
    int* blk_count = reinterpret_cast<int*>(base + L.blk_count);
    int* blk_prefix = reinterpret_cast<int*>(base + L.blk_prefix);
    const int per_task = NOALLOC_CHUNK / NOALLOC_TPB;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n_items;
         i += (long)gridDim.x * blockDim.x) {
        item_task[i] = (int)(i / per_task);
        item_start[i] = (int)(i % per_task) * NOALLOC_TPB;
    }
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t <= n_tasks;
         t += (long)gridDim.x * blockDim.x) {
        src_ptr[t] = (int)t;
        if (t == n_tasks) continue;
        task_tgt[t] = t * NOALLOC_CHUNK;
        task_count[t] = (int)min((long)NOALLOC_CHUNK, n_obs - t * NOALLOC_CHUNK);
        task_origin[3 * t] = task_origin[3 * t + 1] = task_origin[3 * t + 2] = 0.0;
        blk[t] = 0;
        blk_count[t] = n_src;
        blk_prefix[t] = 0;
    }
}

__global__ void noalloc_weight(const double* x, const double* w, double* s, long N, long total)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x)
        s[t] = w[t % N] * x[t];
}

bool on_device(const void* p)
{
    cudaPointerAttributes a{};
    bool dev = p && cudaPointerGetAttributes(&a, p) == cudaSuccess &&
               (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    return dev;
}

}  // namespace

extern "C" int tbem_direct_apply_noalloc(int kernel, const double* kernel_params,
                                         const double* obs_locs, const double* obs_normals,
                                         long n_obs, const double* src_locs,
                                         const double* src_normals, const double* src_weights,
                                         long n_src, const double* x, double* y, int n_rhs,
                                         void* stream)
{
    using namespace tbem;
    try {
        if (kernel < 0 || kernel > 6)
            throw Error(TBEM_ERR_ARG, "tbem_direct_apply_noalloc takes the 3D kernel ids 0..6 "
                                      "only (2D points would need widening, i.e. scratch)");
        if (n_obs < 0 || n_src < 0 || n_rhs <= 0) throw Error(TBEM_ERR_ARG, "bad point count or n_rhs");
        if (kernel_params && on_device(kernel_params))
            throw Error(TBEM_ERR_ARG, "tbem_direct_apply_noalloc: kernel_params is read on the "
                                      "host: pass host memory (or NULL for the defaults)");
        if (n_obs == 0) return TBEM_OK;
        const int R = kernel_dim(kernel);
        const size_t str_bytes = sizeof(double) * (size_t)R * n_src * n_rhs;
        if (str_bytes > NOALLOC_SCRATCH_BYTES - NOALLOC_TASK_BYTES)
            throw Error(TBEM_ERR_ARG, "tbem_direct_apply_noalloc: R * n_src * n_rhs = " +
                                          std::to_string((size_t)R * n_src * n_rhs) +
                                          " exceeds the scratch limit of " +
                                          std::to_string((NOALLOC_SCRATCH_BYTES - NOALLOC_TASK_BYTES) / 8) +
                                          " doubles");
        const long n_tasks = (n_obs + NOALLOC_CHUNK - 1) / NOALLOC_CHUNK;
        const long last = n_obs - (n_tasks - 1) * NOALLOC_CHUNK;
        const long n_items = (n_tasks - 1) * (NOALLOC_CHUNK / NOALLOC_TPB) +
                             (last + NOALLOC_TPB - 1) / NOALLOC_TPB;
        const TaskLayout TL = layout((int)std::min<long>(n_tasks, INT32_MAX),
                                     (int)std::min<long>(n_items, INT32_MAX));
        if (n_items > INT32_MAX || TL.total > NOALLOC_TASK_BYTES)
            throw Error(TBEM_ERR_ARG, "tbem_direct_apply_noalloc: n_obs = " + std::to_string(n_obs) +
                                          " needs more work-item descriptors than the scratch "
                                          "limit allows (about 3 million points)");
        if (n_src > INT32_MAX) throw Error(TBEM_ERR_ARG, "too many sources");
        const bool src_ok = n_src == 0 || (on_device(src_locs) && on_device(src_normals) &&
                                           on_device(src_weights) && on_device(x));
        if (!on_device(obs_locs) || !on_device(obs_normals) || !on_device(y) || !src_ok)
            throw Error(TBEM_ERR_ARG, "tbem_direct_apply_noalloc: every data pointer must be "
                                      "device memory (this entry point copies nothing)");
        unsigned char* base = scratch_address();
        double* str = reinterpret_cast<double*>(base + NOALLOC_TASK_BYTES);
        cudaStream_t s = (cudaStream_t)stream;

        noalloc_fill_tasks<<<(unsigned)std::min<long>((n_items + 255) / 256 + 1, 4096), 256, 0, s>>>(
            base, TL, n_obs, (int)n_src, (int)n_tasks, (int)n_items);
        TBEM_CK(cudaGetLastError());
        const long total = (long)R * n_src * n_rhs;
        if (total > 0) {
            noalloc_weight<<<(unsigned)std::max<long>(1, std::min<long>((total + 255) / 256, 9728)), 256, 0, s>>>(
                x, src_weights, str, n_src, total);
            TBEM_CK(cudaGetLastError());
        }
        const double mu = (kernel_params && R == 3) ? kernel_params[0] : 1.0;
        const double nu = (kernel_params && R == 3) ? kernel_params[1] : 0.25;
        const KParams kp = make_kparams(kernel, mu, nu);
        EvalArgs<double> a{};
        a.item_task = reinterpret_cast<const int*>(base + TL.item_task);
        a.item_start = reinterpret_cast<const int*>(base + TL.item_start);
        a.task_tgt = reinterpret_cast<const long*>(base + TL.task_tgt);
        a.task_tgt_count = reinterpret_cast<const int*>(base + TL.task_count);
        a.task_origin = reinterpret_cast<const double*>(base + TL.task_origin);
        a.task_src_ptr = reinterpret_cast<const int*>(base + TL.src_ptr);
        a.src_blk = reinterpret_cast<const long*>(base + TL.blk);
        a.src_blk_count = reinterpret_cast<const int*>(base + TL.blk_count);
        a.src_blk_prefix = reinterpret_cast<const int*>(base + TL.blk_prefix);
        a.t_xyz = obs_locs;
        a.t_nrm = obs_normals;
        a.s_xyz = src_locs;
        a.s_nrm = src_normals;
        a.s_str = str;
        a.s_n = n_src;
        a.y = y;
        a.y_n = n_obs;
        a.nrhs = n_rhs;
        a.add = 0;
        a.c2 = kp.c2;
        a.scale = kp.scale;
        EvalLaunch L{kernel, false, false, false, (int)n_items};
        for (int r0 = 0; r0 < n_rhs; r0 += (n_rhs - r0 > 1 ? EVAL_NR : 1)) {
            a.rhs0 = r0;
            TBEM_CK(launch_eval<double>(L, a, s));
        }
        return TBEM_OK;
    } catch (...) {
        return tbem::api_status();
    }
}
