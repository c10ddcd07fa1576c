"""Host tests of the autograd routing (no GPU): fmm_apply_sources and
fmm_apply_geometry driven by a dense CPU stand-in with the FMM operator's
method names, against torch's own differentiation of the same dense sum."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
from tbempy import autograd  # noqa: E402


def kernel_matrix(ol, on, sl, sn, sw):
    """A_ij = w_j (1 / r + (n_j - n_i / 2) . d / r^3) / (4 pi), d = x_i - y_j:
    single layer, double layer and half an adjoint double layer, so every
    position, both normals and the weights enter."""
    d = ol[:, None, :] - sl[None, :, :]
    r = torch.linalg.norm(d, dim=-1)
    nd = (d * (sn[None, :, :] - 0.5 * on[:, None, :])).sum(-1)
    return sw[None, :] * (1.0 / r + nd / r ** 3) / (4 * math.pi)


class DenseOp:
    """The operator's apply / transpose / gradient entry points over the dense
    sum above, at fixed points (as an FMMOperator is built at fixed points)."""

    def __init__(self, ol, on, sl, sn, sw):
        self.g = [t.detach().clone() for t in (ol, on, sl, sn, sw)]
        self.calls = {"source": 0, "observation": 0, "adjoint": 0}

    def A(self):
        return kernel_matrix(*self.g)

    def apply(self, x):
        return self.A() @ x

    def apply_adjoint(self, r):
        self.calls["adjoint"] += 1
        return self.A().T @ r

    def _grads(self, x, r, idx):
        # (the backward pass runs with grad mode off; the stand-in uses torch's)
        with torch.enable_grad():
            g = [t.clone().requires_grad_(i in idx) for i, t in enumerate(self.g)]
            L = r @ (kernel_matrix(*g) @ x)
            out = torch.autograd.grad(L, [g[i] for i in idx])
        return dict(zip(idx, out))

    def source_gradients(self, x, r):
        self.calls["source"] += 1
        g = self._grads(x, r, [2, 3, 4])
        return {"src_locs": g[2], "src_normals": g[3], "src_weights": g[4]}

    def observation_gradients(self, x, r):
        self.calls["observation"] += 1
        g = self._grads(x, r, [0, 1])
        return {"obs_locs": g[0], "obs_normals": g[1]}


def inputs(seed):
    rng = np.random.default_rng(seed)
    sl = rng.uniform(0, 1, (40, 3))
    ol = rng.uniform(2, 3, (30, 3))
    sn = rng.normal(size=(40, 3))
    sn /= np.linalg.norm(sn, axis=1)[:, None]
    on = rng.normal(size=(30, 3))
    sw = rng.uniform(0.5, 1.0, 40)
    x = rng.uniform(-1, 1, 40)
    d = rng.normal(size=30)
    return [torch.tensor(a) for a in (ol, on, sl, sn, sw, x, d)]


def test_geometry_gradients_reach_every_input():
    ol, on, sl, sn, sw, x, d = inputs(1)
    op = DenseOp(ol, on, sl, sn, sw)
    leaves = [t.clone().requires_grad_() for t in (ol, on, sl, sn, sw, x)]
    y = autograd.fmm_apply_geometry(op, *leaves)
    (0.5 * ((y - d) ** 2).sum()).backward()
    ref = [t.clone().requires_grad_() for t in (ol, on, sl, sn, sw, x)]
    yr = kernel_matrix(*ref[:5]) @ ref[5]
    (0.5 * ((yr - d) ** 2).sum()).backward()
    for a, b in zip(leaves, ref):
        assert torch.allclose(a.grad, b.grad, rtol=1e-12, atol=1e-14)
    assert op.calls == {"source": 1, "observation": 1, "adjoint": 1}


def test_geometry_computes_only_the_gradients_asked_for():
    ol, on, sl, sn, sw, x, d = inputs(2)
    op = DenseOp(ol, on, sl, sn, sw)
    sl_ = sl.clone().requires_grad_()
    y = autograd.fmm_apply_geometry(op, ol, on, sl_, sn, sw, x)
    (0.5 * ((y - d) ** 2).sum()).backward()
    assert op.calls == {"source": 1, "observation": 0, "adjoint": 0}
    ref = sl.clone().requires_grad_()
    (0.5 * ((kernel_matrix(ol, on, ref, sn, sw) @ x - d) ** 2).sum()).backward()
    assert torch.allclose(sl_.grad, ref.grad, rtol=1e-12, atol=1e-14)


def test_source_geometry_function_matches_dense_differentiation():
    ol, on, sl, sn, sw, x, d = inputs(3)
    op = DenseOp(ol, on, sl, sn, sw)
    leaves = [t.clone().requires_grad_() for t in (sl, sn, sw, x)]
    y = autograd.fmm_apply_sources(op, *leaves)
    (0.5 * ((y - d) ** 2).sum()).backward()
    ref = [t.clone().requires_grad_() for t in (sl, sn, sw, x)]
    (0.5 * ((kernel_matrix(ol, on, *ref[:3]) @ ref[3] - d) ** 2).sum()).backward()
    for a, b in zip(leaves, ref):
        assert torch.allclose(a.grad, b.grad, rtol=1e-12, atol=1e-14)
