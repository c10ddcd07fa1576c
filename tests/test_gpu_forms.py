"""GPU tests of the differentiation form (autograd through the transposed
apply), the FP64 iterative refinement around the precision form, and the
IntegralOperator composition A = G F I + N + C."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cloud(n, seed):
    rng = np.random.default_rng(seed)
    locs = rng.uniform(0, 1, (n, 3))
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    return locs, nrm, rng.uniform(0.5, 1.0, n)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_misfit_gradient_matches_transpose_and_finite_differences(prec):
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD, autograd
    src, sn, w = cloud(400, 1)
    obs, on, _ = cloud(300, 2)
    op = ThreeD.FMMOperator(ThreeD.ElasticDisplacement(1.0, 0.25), obs, on, src, sn, w,
                            ThreeD.FMMConfig(0.3, 296 if prec == "mixed" else 35, 30, 0.05, False),
                            precision=prec)
    rng = np.random.default_rng(3)
    s = torch.tensor(rng.uniform(-1, 1, op.n_cols()), device="cuda", requires_grad=True)
    d = torch.tensor(rng.normal(size=op.n_rows()), device="cuda")
    L = autograd.misfit(op, s, d)
    L.backward()
    g = s.grad.cpu().numpy()
    # against the dense transpose: A^T (A s - d)
    A = op.apply(np.eye(op.n_cols())).T
    r = A @ s.detach().cpu().numpy() - d.cpu().numpy()
    g_dense = A.T @ r
    # the precision form's forward M2L runs on the tensor cores (3xBF16) and its
    # transpose on the FP32 pipes: the two agree to the split's rounding.  The
    # plain form's check-to-equivalent pseudo-inverse (condition ~1e9) turns the
    # 1e-16 differences between its forward and transposed arithmetic into
    # ~1e-10: 1e-9 is the transpose bound there.
    tol = 1e-9 if prec == "fp64" else 2e-5
    assert np.linalg.norm(g - g_dense) <= tol * np.linalg.norm(g_dense)
    # central finite differences on 64 random coordinates.  The loss is exactly
    # quadratic in s, so central differences are exact for any step; a unit
    # step keeps each apply's rounding noise (plain form: ~3e-9 relative, see
    # test_plain_fmm_linearity_floor; precision form: FP32) far below the
    # tolerance
    h = 1.0
    fd_tol = 1e-6 if prec == "fp64" else 2e-5
    s0 = s.detach()
    for j in rng.choice(op.n_cols(), 64, replace=False):
        e = torch.zeros_like(s0)
        e[j] = h
        fd = (autograd.misfit(op, s0 + e, d) - autograd.misfit(op, s0 - e, d)).item() / (2 * h)
        assert abs(fd - g[j]) <= fd_tol * max(1.0, np.abs(g).max())


def test_plain_fmm_linearity_floor():
    """The reference's FMM formulation is linear only up to ~1e-9: its
    pseudo-inverse (condition ~1e9) turns rounding into input-dependent noise.
    Bit-reproducible, but A(x1 + x2) != A x1 + A x2 at that level -- the floor
    of any FP64 residual formed with it."""
    from tbempy import ThreeD, meshes
    locs, nrm, w = meshes.sphere_points(3)
    op = ThreeD.FMMOperator(ThreeD.LaplaceDouble(), locs, nrm, locs, nrm, w,
                            ThreeD.FMMConfig(0.3, 152, 40, 0.05, False), precision="fp64")
    rng = np.random.default_rng(5)
    x1, x2 = rng.uniform(-1, 1, (2, op.n_cols()))
    y1, y2, y12 = op.apply(x1), op.apply(x2), op.apply(x1 + x2)
    nonlin = np.linalg.norm(y12 - y1 - y2) / np.linalg.norm(y12)
    assert nonlin < 1e-7
    assert np.array_equal(op.apply(x1), y1)


def test_refined_gmres_reaches_fp64_residual():
    """Second-kind Laplace system (0.5 I + D) sigma = f on a sphere: the inner
    GMRES runs on the precision-form FMM, the FP64 residual uses the GPU FP64
    direct operator (linear to rounding); the refined solve reaches 1e-10."""
    from tbempy import ThreeD, meshes, solve
    locs, nrm, w = meshes.sphere_points(3)
    cfg = ThreeD.FMMConfig(0.3, 152, 40, 0.05, False)
    K = ThreeD.LaplaceDouble()
    direct = ThreeD.DirectOperator(K, locs, nrm, locs, nrm, w)
    fast = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed")
    A64 = lambda v: 0.5 * v + direct.apply(v)
    A32 = lambda v: 0.5 * v + fast.apply(v)
    f = 1.0 / np.linalg.norm(locs - np.array([0.1, 0.2, 0.3]), axis=1)
    x, hist = solve.refined_solve(A64, A32, f, tol=1e-10, inner_tol=1e-6)
    assert hist[-1][2] <= 1e-10, hist
    assert np.linalg.norm(A64(x) - f) <= 1e-10 * np.linalg.norm(f)
    # the plain FP64 GMRES on the same system, against the same residual
    plain = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="fp64")
    xp, info, _ = solve.gmres(lambda v: 0.5 * v + plain.apply(v), f, restart=50, tol=1e-10)
    assert np.linalg.norm(A64(xp) - f) <= 1e-6 * np.linalg.norm(f)


def test_integral_operator_composition():
    from tbempy import ThreeD
    rng = np.random.default_rng(4)
    locs, nrm, w = cloud(500, 5)
    far = ThreeD.FMMOperator(ThreeD.LaplaceSingle(), locs, nrm, locs, nrm, w,
                             ThreeD.FMMConfig(0.3, 35, 25, 0.05, False))
    n_dof = 200

    def rand_csr(n_rows, n_cols, nnz):
        r = rng.integers(0, n_rows, nnz)
        c = rng.integers(0, n_cols, nnz)
        v = rng.normal(size=nnz)
        D = np.zeros((n_rows, n_cols))
        np.add.at(D, (r, c), v)
        return ThreeD.SparseOperator.csr_from_coo(n_rows, n_cols, r, c, v), D

    interp, I = rand_csr(500, n_dof, 1500)
    galerkin, G = rand_csr(n_dof, 500, 1500)
    near, N = rand_csr(n_dof, n_dof, 800)
    corr, Cm = rand_csr(n_dof, n_dof, 800)
    op = ThreeD.IntegralOperator(near, corr, galerkin, far, interp)
    assert op._h is not None  # the device-side chain (tbem_integral_apply)
    x = rng.normal(size=n_dof)
    expect = G @ far.apply(I @ x) + N @ x + Cm @ x
    assert np.linalg.norm(op.apply(x) - expect) <= 1e-12 * np.linalg.norm(expect)
    assert op.n_rows() == n_dof and op.n_cols() == n_dof
    # several right-hand sides, device tensors in and out.  A batched apply
    # sums in another order than single ones, and the plain form's
    # pseudo-inverse (condition ~1e9) lifts that rounding to ~1e-12: 1e-10
    torch = pytest.importorskip("torch")
    X = rng.normal(size=(3, n_dof))
    Y = op.apply(torch.tensor(X, device="cuda")).cpu().numpy()
    for r in range(3):
        e = G @ far.apply(I @ X[r]) + N @ X[r] + Cm @ X[r]
        assert np.linalg.norm(Y[r] - e) <= 1e-10 * np.linalg.norm(e)
    # shapes that do not chain are refused
    with pytest.raises(Exception):
        ThreeD.IntegralOperator(near, corr, galerkin, far, rand_csr(499, n_dof, 100)[0])


@pytest.mark.parametrize("name", ["ElasticDisplacement", "ElasticTraction", "LaplaceDouble",
                                  "ElasticHypersingular"])
def test_vertex_gradients_match_central_differences(name):
    """Differentiated misfit L = 0.5 ||G(v) s - d||^2 over a bumpy fault's
    vertex coordinates v, observers on the free surface z = 0: the GPU
    kernel-gradient pass (through torch autograd) against FP64 central
    differences (h = 1e-6) on 64 random coordinates."""
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD, autograd, meshes
    v, t, uv = meshes.dipping_fault(12, 45.0)
    v[:, 2] += 0.05 * np.sin(3 * v[:, 0]) * np.cos(2 * v[:, 1])
    rng = np.random.default_rng(3)
    obs = np.column_stack([rng.uniform(-3, 3, 600), rng.uniform(-3, 3, 600), np.zeros(600)])
    on = np.tile([0.0, 0.0, 1.0], (600, 1))
    K = getattr(ThreeD, name)(1.0, 0.25) if name.startswith("Elastic") else ThreeD.LaplaceDouble()
    R = K.tensor_dim
    dev = "cuda"
    V = torch.tensor(v, device=dev, requires_grad=True)
    OL = torch.tensor(obs, device=dev)
    ON = torch.tensor(on, device=dev)
    s = torch.tensor(rng.uniform(-1, 1, R * 3 * len(t)), device=dev)
    d = torch.tensor(rng.normal(size=R * 600) * 1e-3, device=dev)

    def loss(Vt):
        sl, sn, sw = meshes.points_from_mesh_torch(Vt, t)
        y = autograd.direct_apply(K, OL, ON, sl, sn, sw, s)
        return 0.5 * ((y - d) ** 2).sum()

    L = loss(V)
    L.backward()
    # the direct operator is linear to rounding, so a small step is usable here
    g = V.grad.cpu().numpy().ravel()
    h = 1e-6
    flat = v.ravel()
    for k in rng.choice(flat.size, 64, replace=False):
        vp, vm = flat.copy(), flat.copy()
        vp[k] += h
        vm[k] -= h
        with torch.no_grad():
            fd = (loss(torch.tensor(vp.reshape(v.shape), device=dev)) -
                  loss(torch.tensor(vm.reshape(v.shape), device=dev))).item() / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, np.abs(g).max()), (k, fd, g[k])
