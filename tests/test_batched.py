"""The batched form: one operator over many independent meshes
(tbem_fmm_batch_create), every pass covering all meshes in one launch.

Host side (CPU): each mesh's tree is cut from the cube [-1, 1]^3 after the
mesh is centred and scaled, so every mesh's level-l cells are the same
cubes; the task lists never pair cells of different meshes; a mesh's tree
and lists inside the batch equal those of the mesh built alone.

GPU: the batched apply against the FP64 direct sum of every mesh on its
own (the reference applies one mesh and one right-hand side per call,
cpp/fmm.cpp:551-557), in both forms and with 16+ right-hand sides (the wide
evaluation kernels), and its CUDA-graph replay.  Tolerances: the precision
form 2e-6 relative L2 per mesh (the order-152 Laplace bound of the single
operator), the plain form 1e-6.
"""
import numpy as np
import pytest

LISTS = ["p2m", "m2m", "p2p", "m2p", "p2l", "m2l", "l2l", "l2p"]


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def small_batch(n_meshes=5, seed=3, levels=(1, 3), n_rhs=1):
    from tbempy import meshes
    return meshes.sphere_batch(n_meshes=n_meshes, seed=seed, levels=levels, n_rhs=n_rhs)


def test_batch_generator_matches_its_description():
    from tbempy import meshes
    locs, nrm, w, off, x = meshes.sphere_batch(n_meshes=7, seed=2, levels=(2, 3), n_rhs=3)
    assert off[0] == 0 and off[-1] == len(locs) == len(nrm) == len(w) == x.shape[1]
    assert x.shape[0] == 3 and np.all(np.abs(x) <= 1)
    for m in range(7):
        n = off[m + 1] - off[m]
        assert n in (3 * 320, 3 * 1280)
        c = locs[off[m]:off[m + 1]]
        centre = c.mean(axis=0)
        assert np.all(np.abs(centre) <= 100)
        # outward normals
        assert np.all(np.einsum("ij,ij->i", nrm[off[m]:off[m + 1]], c - centre) > 0)


def test_batched_trees_are_cubes_and_lists_stay_within_meshes():
    from tbempy import ThreeD
    locs, nrm, w, off, _ = small_batch()
    cfg = ThreeD.FMMConfig(0.3, 152, 40, 0.05, False)
    op = ThreeD.BatchedFMMOperator(ThreeD.LaplaceDouble(), locs, nrm, w, off, cfg, host_only=True)
    assert op.n_meshes() == len(off) - 1
    t = op.tree(0)
    # every cell of level l is a cube of half width 2^-l (the root's cube [-1, 1]^3)
    assert np.array_equal(t["hw"], np.repeat(2.0 ** -t["level"][:, None], 3, axis=1))
    mesh_of_point = np.searchsorted(off, np.arange(len(locs)), side="right") - 1
    mesh_of_cell = np.array([mesh_of_point[ix[0]] for ix in t["indices"]])
    for ix, m in zip(t["indices"], mesh_of_cell):
        assert np.all(mesh_of_point[ix] == m)
    for kind in ("p2p", "m2l"):
        assert len(op.list(kind)[0]) > 0
    # a host-only operator's construction is its trees and lists alone
    phases = op.setup_times()
    assert [n for n, _ in phases] == ["trees_lists"] and phases[0][1] >= 0
    # a mesh inside the batch has the tree of the same mesh alone (and its
    # lists: next test), so no list pairs cells of two meshes
    for m in range(len(off) - 1):
        sl = slice(off[m], off[m + 1])
        alone = ThreeD.BatchedFMMOperator(ThreeD.LaplaceDouble(), locs[sl], nrm[sl], w[sl],
                                          [0, off[m + 1] - off[m]], cfg, host_only=True)
        ta = alone.tree(0)
        cells = np.nonzero(mesh_of_cell == m)[0]
        for k in ("level", "index", "hw", "n_idx", "n_children"):
            assert np.array_equal(t[k][cells], ta[k]), k
        for ia, ib in zip([t["indices"][c] for c in cells], ta["indices"]):
            assert np.array_equal(ia - off[m], ib)


def test_batched_lists_are_the_meshes_lists_concatenated():
    from tbempy import ThreeD
    locs, nrm, w, off, _ = small_batch(n_meshes=4, seed=5)
    cfg = ThreeD.FMMConfig(0.3, 152, 30, 0.05, False)
    op = ThreeD.BatchedFMMOperator(ThreeD.LaplaceSingle(), locs, nrm, w, off, cfg, host_only=True)
    for kind in LISTS:
        a, b = op.list(kind)
        ea, eb = [], []
        for m in range(len(off) - 1):
            sl = slice(off[m], off[m + 1])
            alone = ThreeD.BatchedFMMOperator(ThreeD.LaplaceSingle(), locs[sl], nrm[sl], w[sl],
                                              [0, off[m + 1] - off[m]], cfg, host_only=True)
            u, v = alone.list(kind)
            ea.append(u)
            eb.append(v)
        assert np.array_equal(a, np.concatenate(ea)), kind
        assert np.array_equal(b, np.concatenate(eb)), kind


def test_batched_create_rejects_bad_offsets():
    from tbempy import ThreeD
    from tbempy._lib import TbemError
    locs, nrm, w, off, _ = small_batch(n_meshes=2)
    cfg = ThreeD.FMMConfig(0.3, 152, 30, 0.05, False)
    for bad in ([1, off[1], off[2]], [0, off[2], off[1]]):
        with pytest.raises(TbemError):
            ThreeD.BatchedFMMOperator(ThreeD.LaplaceDouble(), locs, nrm, w, bad, cfg, host_only=True)
    with pytest.raises(TbemError):  # 2D kernels are refused
        from tbempy import TwoD
        ThreeD.BatchedFMMOperator(TwoD.LaplaceSingle(), locs, nrm, w, off, cfg, host_only=True)


def _direct_per_mesh(K, locs, nrm, w, off, X):
    from tbempy import ThreeD
    out = np.zeros_like(X)
    for m in range(len(off) - 1):
        sl = slice(off[m], off[m + 1])
        d = ThreeD.DirectOperator(K, locs[sl], nrm[sl], locs[sl], nrm[sl], w[sl])
        out[:, sl] = d.apply(np.ascontiguousarray(X[:, sl]))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("prec,n_rhs", [("mixed", 1), ("mixed", 20), ("fp64", 3)])
def test_batched_apply_matches_direct_per_mesh(prec, n_rhs):
    from tbempy import ThreeD
    locs, nrm, w, off, X = small_batch(n_meshes=6, seed=7, levels=(1, 3), n_rhs=n_rhs)
    K = ThreeD.LaplaceDouble()
    cfg = ThreeD.FMMConfig(0.3, 152, 40, 0.05, False)
    op = ThreeD.BatchedFMMOperator(K, locs, nrm, w, off, cfg, precision=prec)
    Y = op.apply(X)
    exact = _direct_per_mesh(K, locs, nrm, w, off, X)
    tol = 2e-6 if prec == "mixed" else 1e-6
    for m in range(len(off) - 1):
        sl = slice(off[m], off[m + 1])
        err = rel(Y[:, sl], exact[:, sl])
        assert err < tol, (m, err)


@pytest.mark.gpu
def test_batched_single_layer_scales_with_the_mesh():
    """LaplaceSingle (degree -1): the weights are rescaled by the mesh size;
    the result must still be the unscaled operator's."""
    from tbempy import ThreeD
    locs, nrm, w, off, X = small_batch(n_meshes=4, seed=11, levels=(2, 3), n_rhs=2)
    K = ThreeD.LaplaceSingle()
    op = ThreeD.BatchedFMMOperator(K, locs, nrm, w, off, ThreeD.FMMConfig(0.3, 152, 40, 0.05, False))
    Y = op.apply(X)
    exact = _direct_per_mesh(K, locs, nrm, w, off, X)
    for m in range(len(off) - 1):
        sl = slice(off[m], off[m + 1])
        assert rel(Y[:, sl], exact[:, sl]) < 2e-6


@pytest.mark.gpu
def test_batched_graph_replay():
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD
    locs, nrm, w, off, X = small_batch(n_meshes=5, seed=13, levels=(1, 2), n_rhs=16)
    op = ThreeD.BatchedFMMOperator(ThreeD.LaplaceDouble(), locs, nrm, w, off,
                                   ThreeD.FMMConfig(0.3, 152, 30, 0.05, False))
    x = torch.tensor(X, device="cuda")
    y = torch.zeros_like(x)
    g = ThreeD.FMMGraph([op], [x], [y], n_rhs=16)
    x.uniform_(-1, 1)
    y.zero_()
    g.launch()
    torch.cuda.synchronize()
    ref = op.apply(x)
    assert (torch.linalg.norm(y - ref) / torch.linalg.norm(ref)).item() < 1e-6
