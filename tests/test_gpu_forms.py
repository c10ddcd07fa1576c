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


@pytest.mark.parametrize("prec", ["mixed", "fp64_compressed"])
@pytest.mark.parametrize("name", ["LaplaceSingle", "LaplaceDouble", "ElasticDisplacement",
                                  "ElasticTraction"])
@pytest.mark.parametrize("distinct", [False, True])
def test_fmm_source_gradients_match_the_direct_pass(name, distinct, prec):
    """tbem_fmm_source_gradients (the FMM's transposed passes with the
    kernel's derivatives) against the direct kernel-gradient pass: positions,
    normals and weights of the sources, to the form's approximation error."""
    from tbempy import ThreeD
    src, sn, w = cloud(600, 11)
    obs, on = (src, sn) if not distinct else cloud(500, 12)[:2]
    K = ThreeD.ElasticDisplacement(1.0, 0.25) if name == "ElasticDisplacement" else \
        ThreeD.ElasticTraction(1.0, 0.25) if name == "ElasticTraction" else getattr(ThreeD, name)()
    op = ThreeD.FMMOperator(K, obs, on, src, sn, w, ThreeD.FMMConfig(0.3, 296, 30, 0.05, False),
                            precision=prec)
    rng = np.random.default_rng(13)
    x = rng.uniform(-1, 1, op.n_cols())
    r = rng.uniform(-1, 1, op.n_rows())
    op.apply(rng.uniform(-1, 1, op.n_cols()))  # leave other states in the work buffers
    g = op.source_gradients(x, r)
    gd = ThreeD.direct_gradients(K, obs, on, src, sn, w, x, r)
    tol = 2e-5 if prec == "mixed" else 2e-6
    for k in ("src_locs", "src_weights") + (("src_normals",) if name in ("LaplaceDouble", "ElasticTraction") else ()):
        err = np.linalg.norm(g[k] - gd[k]) / np.linalg.norm(gd[k])
        assert err < tol, (k, err)


@pytest.mark.parametrize("prec", ["mixed", "fp64_compressed"])
@pytest.mark.parametrize("name", ["LaplaceSingle", "LaplaceDouble", "ElasticAdjointTraction",
                                  "ElasticHypersingular"])
@pytest.mark.parametrize("distinct", [False, True])
def test_fmm_observation_gradients_match_the_direct_pass(name, distinct, prec):
    """tbem_fmm_observation_gradients (the passes that reach observation
    points, with the kernel's derivatives) against the direct
    kernel-gradient pass: positions of the observation points and, for the
    kernels with an observation normal, the normals."""
    from tbempy import ThreeD
    src, sn, w = cloud(600, 11)
    obs, on = (src, sn) if not distinct else cloud(500, 12)[:2]
    K = ThreeD.ElasticAdjointTraction(1.0, 0.25) if name == "ElasticAdjointTraction" else \
        ThreeD.ElasticHypersingular(1.0, 0.25) if name == "ElasticHypersingular" else getattr(ThreeD, name)()
    op = ThreeD.FMMOperator(K, obs, on, src, sn, w, ThreeD.FMMConfig(0.3, 296, 30, 0.05, False),
                            precision=prec)
    rng = np.random.default_rng(17)
    x = rng.uniform(-1, 1, op.n_cols())
    r = rng.uniform(-1, 1, op.n_rows())
    op.apply_adjoint(rng.uniform(-1, 1, op.n_rows()))  # leave other states in the work buffers
    g = op.observation_gradients(x, r)
    gd = ThreeD.direct_gradients(K, obs, on, src, sn, w, x, r)
    tol = 2e-5 if prec == "mixed" else 2e-6
    keys = ("obs_locs",) + (("obs_normals",) if name.startswith("Elastic") else ())
    for k in keys:
        err = np.linalg.norm(g[k] - gd[k]) / np.linalg.norm(gd[k])
        assert err < tol, (k, err)
    if not name.startswith("Elastic"):
        assert np.all(g["obs_normals"] == 0.0)


def test_fmm_geometry_gradient_through_autograd():
    """fmm_apply_geometry: the misfit's gradient with respect to mesh vertices
    that place both the sources and the observation points (pushed off the
    surface along the normals) through the FMM's source and observation
    gradients equals the direct kernel-gradient pass's."""
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD, autograd, meshes
    v, t, _, _, _, _, _ = meshes.misfit_workload(n=12, n_obs=400)
    K = ThreeD.ElasticAdjointTraction(1.0, 0.25)
    sl, sn, sw = meshes.points_from_mesh(v, t)
    ol, on = sl + 0.05 * sn, sn
    op = ThreeD.FMMOperator(K, ol, on, sl, sn, sw, ThreeD.FMMConfig(0.3, 296, 30, 0.05, False),
                            precision="mixed")
    s = torch.tensor(np.random.default_rng(4).uniform(-1, 1, op.n_cols()), device="cuda")
    d = torch.tensor(np.random.default_rng(5).normal(size=op.n_rows()), device="cuda")
    grads = []
    for use_fmm in (True, False):
        V = torch.tensor(v, device="cuda", requires_grad=True)
        a, b, c = meshes.points_from_mesh_torch(V, t)
        o = a + 0.05 * b
        y = (autograd.fmm_apply_geometry(op, o, b, a, b, c, s) if use_fmm
             else autograd.direct_apply(K, o, b, a, b, c, s))
        (0.5 * ((y - d) ** 2).sum()).backward()
        grads.append(V.grad.cpu().numpy())
    err = np.linalg.norm(grads[0] - grads[1]) / np.linalg.norm(grads[1])
    assert err < 2e-5, err


def test_fmm_vertex_gradient_through_autograd():
    """fmm_apply_sources: the misfit's gradient with respect to mesh vertices
    (points, normals and weights from the vertices by torch) through the
    FMM's source gradients equals the direct kernel-gradient pass's."""
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD, autograd, meshes
    v, t, obs, on, _, _, _ = meshes.misfit_workload(n=12, n_obs=400)
    sl, sn, sw = meshes.points_from_mesh(v, t)
    K = ThreeD.ElasticDisplacement(1.0, 0.25)
    op = ThreeD.FMMOperator(K, obs, on, sl, sn, sw, ThreeD.FMMConfig(0.3, 296, 30, 0.05, False),
                            precision="mixed")
    s = torch.tensor(np.random.default_rng(4).uniform(-1, 1, op.n_cols()), device="cuda")
    d = torch.tensor(np.random.default_rng(5).normal(size=op.n_rows()), device="cuda")
    OL, ON = torch.tensor(obs, device="cuda"), torch.tensor(on, device="cuda")
    grads = []
    for use_fmm in (True, False):
        V = torch.tensor(v, device="cuda", requires_grad=True)
        a, b, c = meshes.points_from_mesh_torch(V, t)
        y = (autograd.fmm_apply_sources(op, a, b, c, s) if use_fmm
             else autograd.direct_apply(K, OL, ON, a, b, c, s))
        (0.5 * ((y - d) ** 2).sum()).backward()
        grads.append(V.grad.cpu().numpy())
    err = np.linalg.norm(grads[0] - grads[1]) / np.linalg.norm(grads[1])
    assert err < 2e-5, err


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


@pytest.mark.parametrize("name,order", [("LaplaceSingle", 152), ("LaplaceDouble", 296),
                                        ("ElasticTraction", 296)])
def test_fp64_compressed_form_is_linear_and_accurate(name, order):
    """The FP64 compressed form (the precision form's operators applied in
    FP64): against the FP64 direct sum at the precision form's bound (2e-6);
    linear to rounding, A(x1 + x2) = A x1 + A x2 to 1e-13 (the plain form's
    floor is ~1e-9); its transpose satisfies <A x, z> = <x, A^T z> to 1e-13;
    and the FP32 precision form agrees with it to 2e-6."""
    from tbempy import ThreeD, meshes
    locs, nrm, w = meshes.sphere_points(3)
    K = getattr(ThreeD, name)(1.0, 0.25) if name.startswith("Elastic") else getattr(ThreeD, name)()
    cfg = ThreeD.FMMConfig(0.3, order, 40, 0.05, False)
    op = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="fp64_compressed")
    rng = np.random.default_rng(6)
    x1, x2 = rng.uniform(-1, 1, (2, op.n_cols()))
    y1, y2, y12 = op.apply(x1), op.apply(x2), op.apply(x1 + x2)
    assert np.linalg.norm(y12 - y1 - y2) <= 1e-13 * np.linalg.norm(y12)
    exact = ThreeD.DirectOperator(K, locs, nrm, locs, nrm, w).apply(x1)
    assert np.linalg.norm(y1 - exact) <= 2e-6 * np.linalg.norm(exact)
    z = rng.uniform(-1, 1, op.n_rows())
    lhs, rhs = float(y1 @ z), float(x1 @ op.apply_adjoint(z))
    assert abs(lhs - rhs) <= 1e-13 * np.linalg.norm(y1) * np.linalg.norm(z)
    mixed = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed")
    assert np.linalg.norm(mixed.apply(x1) - y1) <= 2e-6 * np.linalg.norm(y1)
    X = np.stack([x1, x2, x1 - x2])
    assert np.linalg.norm(op.apply(X)[2] - (y1 - y2)) <= 1e-13 * np.linalg.norm(y1 - y2)


def test_refined_gmres_with_an_fmm_fp64_residual():
    """The refinement's FP64 residual through the FP64 compressed form -- an
    O(N) operator linear to rounding -- instead of the O(N^2) direct sum: the
    refined solve (inner GMRES on the FP32 / tensor-core precision form)
    reaches 1e-10 against that operator, and the solution satisfies the
    direct operator's system to the FMM's own accuracy."""
    from tbempy import ThreeD, meshes, solve
    locs, nrm, w = meshes.sphere_points(3)
    cfg = ThreeD.FMMConfig(0.3, 152, 40, 0.05, False)
    K = ThreeD.LaplaceDouble()
    f64 = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="fp64_compressed")
    fast = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed")
    A64 = lambda v: 0.5 * v + f64.apply(v)
    A32 = lambda v: 0.5 * v + fast.apply(v)
    f = 1.0 / np.linalg.norm(locs - np.array([0.1, 0.2, 0.3]), axis=1)
    x, hist = solve.refined_solve(A64, A32, f, tol=1e-10, inner_tol=1e-6)
    assert hist[-1][2] <= 1e-10, hist
    assert np.linalg.norm(A64(x) - f) <= 1e-10 * np.linalg.norm(f)
    direct = ThreeD.DirectOperator(K, locs, nrm, locs, nrm, w)
    assert np.linalg.norm(0.5 * x + direct.apply(x) - f) <= 1e-5 * np.linalg.norm(f)


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


def test_misfit_workload_at_size():
    """The differentiated workload at its stated size: a 64 x 64-quad bumpy
    fault (8,192 triangles, 24,576 points), 16,384 observers on z = 0,
    L = 0.5 ||G s - d||^2 with the elastic displacement kernel and
    d = G s2 + N(0, 1e-3).

    * dL/ds through the precision-form FMM and its transposed apply (torch
      autograd) against the FP64 direct operator's transpose,
      G^T (G s - d) (the kernel-gradient pass's dL/dx): 2e-6 relative L2
      (the FMM's own error against the direct sum);
    * the same gradient against FP64 central differences (h = 1e-6) of the
      direct loss on 64 random slip coordinates: 2e-6 of the largest entry;
    * dL/d(vertex coordinates) through the kernel-gradient pass against FP64
      central differences (h = 1e-6) on 64 random coordinates: 1e-6 of the
      largest entry."""
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD, autograd, meshes
    v, t, obs, on, s_np, s2_np, noise = meshes.misfit_workload()
    assert len(t) == 8192 and len(obs) == 16384
    K = ThreeD.ElasticDisplacement(1.0, 0.25)
    dev = "cuda"
    sl, sn, sw = meshes.points_from_mesh(v, t)
    assert len(sl) == 24576
    D = ThreeD.DirectOperator(K, obs, on, sl, sn, sw)
    d = torch.tensor(D.apply(s2_np) + noise, device=dev)
    s = torch.tensor(s_np, device=dev)
    op = ThreeD.FMMOperator(K, obs, on, sl, sn, sw, ThreeD.FMMConfig(0.3, 296, 64, 0.05, False),
                            precision="mixed")
    sg = s.clone().requires_grad_(True)
    autograd.misfit(op, sg, d).backward()
    g = sg.grad.cpu().numpy()
    r = D.apply(s_np) - d.cpu().numpy()
    gd = ThreeD.direct_gradients(K, obs, on, sl, sn, sw, s_np, r)["x"]
    gd = np.asarray(gd.cpu() if hasattr(gd, "cpu") else gd).ravel()
    assert np.linalg.norm(g - gd) <= 2e-6 * np.linalg.norm(gd), np.linalg.norm(g - gd) / np.linalg.norm(gd)
    rng = np.random.default_rng(31)
    h = 1e-6

    def direct_loss(x):
        y = D.apply(x) - d.cpu().numpy()
        return 0.5 * float(y @ y)

    for j in rng.choice(len(s_np), 64, replace=False):
        e = np.zeros_like(s_np)
        e[j] = h
        fd = (direct_loss(s_np + e) - direct_loss(s_np - e)) / (2 * h)
        assert abs(fd - g[j]) <= 2e-6 * np.abs(gd).max(), (j, fd, g[j])
    # vertex coordinates through the kernel-gradient pass
    V = torch.tensor(v, device=dev, requires_grad=True)
    OL = torch.tensor(obs, device=dev)
    ON = torch.tensor(on, device=dev)

    def loss(Vt):
        a, b, c = meshes.points_from_mesh_torch(Vt, t)
        y = autograd.direct_apply(K, OL, ON, a, b, c, s)
        return 0.5 * ((y - d) ** 2).sum()

    loss(V).backward()
    gv = V.grad.cpu().numpy().ravel()
    flat = v.ravel()
    for k in rng.choice(flat.size, 64, replace=False):
        vp, vm = flat.copy(), flat.copy()
        vp[k] += h
        vm[k] -= h
        with torch.no_grad():
            fd = (loss(torch.tensor(vp.reshape(v.shape), device=dev)) -
                  loss(torch.tensor(vm.reshape(v.shape), device=dev))).item() / (2 * h)
        assert abs(fd - gv[k]) <= 1e-6 * max(1.0, np.abs(gv).max()), (k, fd, gv[k])


def test_exterior_dirichlet_solve_plain_and_refined():
    """The full-solve workload at a reduced size: the bumpy sphere subdivided
    4 times (15,360 points), the exterior Laplace Dirichlet problem with the
    data of 10 interior unit charges, as the second-kind combined-layer
    system (1/2 I - D + S) mu = g, FMM order 296, MAC 0.3, 64 points per leaf.
    * the FP64 solve -- GMRES(50) on the FP64 compressed operators -- reaches
      1e-10 relative residual;
    * the refined solve -- inner GMRES on the precision form (FP32 / tensor
      cores), FP64 residuals through the FP64 compressed operators --
      reaches the same 1e-10, and the two solutions agree to 1e-9;
    * the field -D mu + S mu at exterior points matches the charges' potential
      to the discretisation's accuracy (5e-2: one-point-per-node quadrature)."""
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD, meshes, solve
    v, t = meshes.bumpy_sphere(4)
    locs, nrm, w = meshes.points_from_mesh(v, t)
    q = meshes.interior_charges()
    g = sum(1.0 / (4 * np.pi * np.linalg.norm(locs - p, axis=1)) for p in q)
    cfg = ThreeD.FMMConfig(0.3, 296, 64, 0.05, False)
    ops = {}
    for prec in ("fp64_compressed", "mixed"):
        ops[prec] = [ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision=prec)
                     for K in (ThreeD.LaplaceSingle(), ThreeD.LaplaceDouble())]
    A64 = solve.exterior_dirichlet_system(ops["fp64_compressed"][0].apply, ops["fp64_compressed"][1].apply)
    A32 = solve.exterior_dirichlet_system(ops["mixed"][0].apply, ops["mixed"][1].apply)
    gt = torch.tensor(g, device="cuda")
    x64, info, its = solve.gmres(A64, gt, restart=50, tol=1e-10)
    assert info == 0
    assert (torch.linalg.norm(A64(x64) - gt) / torch.linalg.norm(gt)).item() <= 1e-10
    xr, hist = solve.refined_solve(A64, A32, gt, tol=1e-10, inner_tol=1e-6)
    assert hist[-1][2] <= 1e-10, hist
    assert (torch.linalg.norm(xr - x64) / torch.linalg.norm(x64)).item() <= 1e-9
    rng = np.random.default_rng(8)
    d = rng.normal(size=(1000, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    X = d * rng.uniform(2.0, 3.0, 1000)[:, None]
    XN = np.tile([0.0, 0.0, 1.0], (1000, 1))
    mu = xr.cpu().numpy()
    u = (-ThreeD.DirectOperator(ThreeD.LaplaceDouble(), X, XN, locs, nrm, w).apply(mu)
         + ThreeD.DirectOperator(ThreeD.LaplaceSingle(), X, XN, locs, nrm, w).apply(mu))
    exact = sum(1.0 / (4 * np.pi * np.linalg.norm(X - p, axis=1)) for p in q)
    assert np.linalg.norm(u - exact) <= 5e-2 * np.linalg.norm(exact)
