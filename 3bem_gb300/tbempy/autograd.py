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


def misfit(op, s, d):
    """L = 0.5 ||A s - d||^2 (the differentiated workload's loss)."""
    r = fmm_apply(op, s) - d
    return 0.5 * (r * r).sum()
