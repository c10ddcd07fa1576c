"""CUDA-graph capture of operator applies (tbem_fmm_graph_*): one graph
launch replays the applies of several operators on different meshes, reading
the inputs' current contents at every replay."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def meshes_and_ops(torch, n_rhs):
    from tbempy import ThreeD, meshes
    rng = np.random.default_rng(50)
    ops, xs, ys, precs = [], [], [], []
    for i, (sub, prec) in enumerate([(1, "fp64"), (2, "fp64"), (2, "mixed"), (3, "mixed")]):
        v, t = meshes.icosphere(sub, radius=1.0 + 0.3 * i, center=(3.0 * i, 0.0, 0.0))
        locs, nrm, w = meshes.points_from_mesh(v, t)
        cfg = ThreeD.FMMConfig(0.3, 35 if prec == "fp64" else 152, 20, 0.05, False)
        op = ThreeD.FMMOperator(ThreeD.LaplaceDouble(), locs, nrm, locs, nrm, w, cfg, precision=prec)
        ops.append(op)
        precs.append(prec)
        xs.append(torch.tensor(rng.uniform(-1, 1, (n_rhs, op.n_cols())), device="cuda"))
        ys.append(torch.zeros((n_rhs, op.n_rows()), dtype=torch.float64, device="cuda"))
    return ops, xs, ys, precs


def test_graph_replays_the_applies_of_many_meshes():
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD
    ops, xs, ys, precs = meshes_and_ops(torch, 2)
    g = ThreeD.FMMGraph(ops, xs, ys, n_rhs=2)
    for _ in range(2):
        for x in xs:
            x.uniform_(-1, 1)  # new inputs: the replay reads the buffers again
        for y in ys:
            y.zero_()
        g.launch()
        torch.cuda.synchronize()
        for op, x, y, prec in zip(ops, xs, ys, precs):
            ref = op.apply(x)
            if prec == "fp64":
                # the plain form is deterministic: the replay is bit-identical
                assert torch.equal(y, ref)
            else:
                assert (torch.linalg.norm(y - ref) / torch.linalg.norm(ref)).item() < 1e-6


def test_graph_of_transposed_applies():
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD
    ops, xs, ys, precs = meshes_and_ops(torch, 1)
    op = ops[1]
    z = torch.rand(op.n_rows(), dtype=torch.float64, device="cuda")
    w = torch.zeros(op.n_cols(), dtype=torch.float64, device="cuda")
    g = ThreeD.FMMGraph([op], [z], [w], adjoint=True)
    w.zero_()
    g.launch()
    torch.cuda.synchronize()
    assert torch.equal(w, op.apply_adjoint(z))


def test_graph_rejects_host_buffers():
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD, _lib
    ops, xs, ys, precs = meshes_and_ops(torch, 1)
    op = ops[0]
    with pytest.raises(_lib.TbemError):
        ThreeD.FMMGraph([op], [torch.zeros(op.n_cols(), dtype=torch.float64)],
                        [torch.zeros(op.n_rows(), dtype=torch.float64)])
