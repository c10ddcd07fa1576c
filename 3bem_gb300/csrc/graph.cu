// CUDA-graph capture of operator applies: the batching form's single launch.
//
// A graph holds the applies of one or several operators (for instance one per
// mesh of a batch) between fixed device buffers.  The operators are spread
// over up to eight parallel branches, so small independent meshes run side by
// side; one cudaGraphLaunch replays everything, without the per-kernel host
// launch cost.  The applies are the ordinary ones (Plan::apply), captured:
// a first, uncaptured apply of every operator sizes its work buffers and
// builds the tile tables of this right-hand-side count, so the captured
// applies make no allocation and no synchronous copy.
#include <algorithm>
#include <string>
#include <vector>

#include "handle.h"

struct TbemGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap = nullptr;                 // capture / default launch stream
    std::vector<cudaStream_t> branch;           // parallel branches
    std::vector<cudaEvent_t> joins;
    cudaEvent_t fork = nullptr;
    std::vector<TbemFmm*> ops;                  // not owned
    int device = 0;
    ~TbemGraph()
    {
        // released on the device they were made on, the caller's given back
        int prev = -1;
        const bool own = cudaGetDevice(&prev) == cudaSuccess && prev != device &&
                         cudaSetDevice(device) == cudaSuccess;
        cudaGetLastError();
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (auto e : joins) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        for (auto b : branch) cudaStreamDestroy(b);
        if (cap) cudaStreamDestroy(cap);
        if (own) cudaSetDevice(prev);
    }
};

namespace tbem {

namespace {

bool on_device(const void* p)
{
    cudaPointerAttributes a{};
    const bool dev = p && cudaPointerGetAttributes(&a, p) == cudaSuccess &&
                     (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    return dev;
}

}  // namespace

void graph_build(TbemGraph& g, TbemFmm* const* ops, int n_ops, const double* const* x,
                 double* const* y, int n_rhs, bool adjoint)
{
    if (n_ops <= 0 || !ops || !x || !y) throw Error(TBEM_ERR_ARG, "no operators to capture");
    if (n_rhs <= 0) throw Error(TBEM_ERR_ARG, "n_rhs must be > 0");
    const int dev = ops[0] ? ops[0]->plan.opt.device : 0;
    for (int i = 0; i < n_ops; i++) {
        if (!ops[i]) throw Error(TBEM_ERR_ARG, "null operator");
        const Plan& p = ops[i]->plan;
        if (p.opt.host_only) throw Error(TBEM_ERR_STATE, "operator was built with host_only");
        if (p.opt.device != dev) throw Error(TBEM_ERR_ARG, "operators on different devices");
        if (p.timing) throw Error(TBEM_ERR_STATE, "phase timing is on: turn it off before capturing");
        const long n_in = (long)p.R * (adjoint ? p.n_obs : p.n_src);
        const long n_out = (long)p.R * (adjoint ? p.n_src : p.n_obs);
        if ((n_in > 0 && !on_device(x[i])) || (n_out > 0 && !on_device(y[i])))
            throw Error(TBEM_ERR_ARG, "a graph replays fixed addresses: inputs and outputs must be device memory");
    }
    g.device = dev;
    DeviceGuard guard(dev);
    TBEM_CK(cudaStreamCreateWithFlags(&g.cap, cudaStreamNonBlocking));
    const int nb = std::min(n_ops, 8);
    g.branch.resize(nb);
    g.joins.resize(nb);
    for (int b = 0; b < nb; b++) {
        TBEM_CK(cudaStreamCreateWithFlags(&g.branch[b], cudaStreamNonBlocking));
        TBEM_CK(cudaEventCreateWithFlags(&g.joins[b], cudaEventDisableTiming));
    }
    TBEM_CK(cudaEventCreateWithFlags(&g.fork, cudaEventDisableTiming));
    // the uncaptured first applies: buffers and tile tables for n_rhs
    for (int i = 0; i < n_ops; i++) ops[i]->plan.apply(x[i], y[i], n_rhs, g.cap, adjoint);
    TBEM_CK(cudaStreamSynchronize(g.cap));
    TBEM_CK(cudaStreamBeginCapture(g.cap, cudaStreamCaptureModeThreadLocal));
    try {
        TBEM_CK(cudaEventRecord(g.fork, g.cap));
        for (int b = 0; b < nb; b++) TBEM_CK(cudaStreamWaitEvent(g.branch[b], g.fork, 0));
        for (int i = 0; i < n_ops; i++) ops[i]->plan.apply(x[i], y[i], n_rhs, g.branch[i % nb], adjoint);
        for (int b = 0; b < nb; b++) {
            TBEM_CK(cudaEventRecord(g.joins[b], g.branch[b]));
            TBEM_CK(cudaStreamWaitEvent(g.cap, g.joins[b], 0));
        }
    } catch (...) {
        cudaGraph_t broken = nullptr;
        cudaStreamEndCapture(g.cap, &broken);
        if (broken) cudaGraphDestroy(broken);
        cudaGetLastError();
        throw;
    }
    TBEM_CK(cudaStreamEndCapture(g.cap, &g.graph));
    TBEM_CK(cudaGraphInstantiate(&g.exec, g.graph, 0));
    g.ops.assign(ops, ops + n_ops);
}

TbemGraph* graph_new() { return new TbemGraph(); }
void graph_delete(TbemGraph* g) { delete g; }

void graph_launch(TbemGraph& g, cudaStream_t s)
{
    for (TbemFmm* op : g.ops) {
        if (op->plan.flags_raised())
            throw Error(TBEM_ERR_TIMEOUT, "a bounded device wait of an earlier replay gave up");
    }
    DeviceGuard guard(g.device);
    TBEM_CK(cudaGraphLaunch(g.exec, s ? s : g.cap));
}

}  // namespace tbem
