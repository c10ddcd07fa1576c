// The opaque operator handle of the C ABI (include/tbem_gpu.h) and the
// graph handle built on it.
#pragma once
#include <vector>

#include "plan.h"

struct TbemFmm {
    tbem::Plan plan;
};

struct TbemGraph;

namespace tbem {
void graph_build(TbemGraph& g, TbemFmm* const* ops, int n_ops, const double* const* x,
                 double* const* y, int n_rhs, bool adjoint);
void graph_launch(TbemGraph& g, cudaStream_t s);
TbemGraph* graph_new();
void graph_delete(TbemGraph* g);
}  // namespace tbem
