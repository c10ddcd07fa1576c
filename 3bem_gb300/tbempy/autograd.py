"""torch.autograd wrapper of the operator apply (the differentiation form).

``fmm_apply(op, x)`` returns ``op.apply(x)`` for a float64 CUDA tensor and
back-propagates with the operator's exact transpose
(``tbem_fmm_apply_adjoint``: the FMM passes transposed and run in reverse
order), so gradients of any loss with respect to the densities cost one
transposed apply.  Nothing is stored between the forward and the backward
pass beyond the operator itself: the expansions are recomputed.
"""
import torch


class _OperatorApply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, op):
        ctx.op = op
        return op.apply(x.contiguous())

    @staticmethod
    def backward(ctx, grad):
        return ctx.op.apply_adjoint(grad.contiguous()), None


def fmm_apply(op, x):
    """Differentiable y = A x (A: an FMMOperator; x: float64 CUDA tensor,
    [n_cols] or [n_rhs, n_cols])."""
    if not hasattr(op, "apply_adjoint"):
        raise TypeError("the operator has no transposed apply")
    return _OperatorApply.apply(x, op)


class _SourceGeometryApply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, src_locs, src_normals, src_weights, x, op):
        ctx.op = op
        ctx.save_for_backward(x)
        return op.apply(x.contiguous())

    @staticmethod
    def backward(ctx, grad):
        (x,) = ctx.saved_tensors
        g = ctx.op.source_gradients(x.detach().contiguous(), grad.contiguous())
        gx = ctx.op.apply_adjoint(grad.contiguous())
        return g["src_locs"], g["src_normals"], g["src_weights"], gx, None


def fmm_apply_sources(op, src_locs, src_normals, src_weights, x):
    """Differentiable y = A x whose gradients also reach the source geometry.

    ``op`` is an FMMOperator (a compressed form) built at the values of
    ``src_locs`` [n, 3], ``src_normals`` [n, 3] and ``src_weights`` [n]
    (float64 CUDA tensors, e.g. computed from mesh vertices that require
    grad); x is the density [n_cols].  The backward pass runs the operator's
    transposed apply for x and ``source_gradients`` (the FMM's transposed
    passes with the kernel's derivatives) for the geometry: O(N), where the
    direct kernel-gradient pass (``direct_apply``) is O(N M)."""
    return _SourceGeometryApply.apply(src_locs, src_normals, src_weights, x, op)


class _GeometryApply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, obs_locs, obs_normals, src_locs, src_normals, src_weights, x, op):
        ctx.op = op
        ctx.save_for_backward(x)
        return op.apply(x.contiguous())

    @staticmethod
    def backward(ctx, grad):
        (x,) = ctx.saved_tensors
        need = ctx.needs_input_grad
        xd, gd = x.detach().contiguous(), grad.contiguous()
        go = {"obs_locs": None, "obs_normals": None}
        gs = {"src_locs": None, "src_normals": None, "src_weights": None}
        if need[0] or need[1]:
            go = ctx.op.observation_gradients(xd, gd)
        if need[2] or need[3] or need[4]:
            gs = ctx.op.source_gradients(xd, gd)
        gx = ctx.op.apply_adjoint(gd) if need[5] else None
        return (go["obs_locs"], go["obs_normals"], gs["src_locs"], gs["src_normals"],
                gs["src_weights"], gx, None)


def fmm_apply_geometry(op, obs_locs, obs_normals, src_locs, src_normals, src_weights, x):
    """Differentiable y = A x whose gradients reach both point sets.

    As ``fmm_apply_sources``, with the observation points' positions and
    normals [n_obs, 3] as inputs too: their gradients come from
    ``observation_gradients`` (one forward apply, then the passes that reach
    observation points with the kernel's derivatives).  Only the gradients
    that are needed are computed."""
    return _GeometryApply.apply(obs_locs, obs_normals, src_locs, src_normals, src_weights, x, op)


def misfit(op, s, d):
    """L = 0.5 ||A s - d||^2 (the differentiated workload's loss)."""
    r = fmm_apply(op, s) - d
    return 0.5 * (r * r).sum()


class _DirectApply(torch.autograd.Function):
    """y = A x with A_ij = w_j K(x_i, y_j; n_i, n_j), differentiable in the
    densities and in every point position, normal and weight."""

    @staticmethod
    def forward(ctx, obs_locs, obs_normals, src_locs, src_normals, src_weights, x, K):
        from .ThreeD import DirectOperator
        ctx.K = K
        ctx.save_for_backward(obs_locs, obs_normals, src_locs, src_normals, src_weights, x)
        op = DirectOperator(K, obs_locs.detach().cpu().numpy(), obs_normals.detach().cpu().numpy(),
                            src_locs.detach().cpu().numpy(), src_normals.detach().cpu().numpy(),
                            src_weights.detach().cpu().numpy())
        return op.apply(x.detach().contiguous())

    @staticmethod
    def backward(ctx, grad):
        from .ThreeD import direct_gradients
        ol, on, sl, sn, sw, x = ctx.saved_tensors
        g = direct_gradients(ctx.K, ol.detach(), on.detach(), sl.detach(), sn.detach(), sw.detach(),
                             x.detach(), grad.contiguous())
        return (g["obs_locs"], g["obs_normals"], g["src_locs"], g["src_normals"],
                g["src_weights"], g["x"], None)


def direct_apply(K, obs_locs, obs_normals, src_locs, src_normals, src_weights, x):
    """Differentiable direct (FP64) operator apply on the GPU; all inputs
    float64 CUDA tensors ([n,3] points/normals, [n] weights, [C n_src] x)."""
    return _DirectApply.apply(obs_locs, obs_normals, src_locs, src_normals, src_weights, x, K)
