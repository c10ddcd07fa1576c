"""GPU parity of the FMM apply against the oracle (CPU restatement of the
reference KIFMM) and against the FP64 direct sum.

Tolerances (written here, checked below):
  * plain FP64 form vs oracle with identical check-to-equivalent operators:
    1e-10 relative L2 (the reference's own FMM is the target; the operators
    are injected so that only the apply is compared);
  * plain FP64 form with its own cuSOLVER operators vs the reference's
    fixtures: max(1e-10, 10 x the reference's one-ulp conditioning floor of
    each case);
  * precision form vs FP64 direct sum at the workload orders: 2e-6.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

KERNELS = ["LaplaceSingle", "LaplaceDouble", "ElasticDisplacement", "ElasticTraction",
           "ElasticAdjointTraction", "ElasticHypersingular"]


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def cloud(n, seed):
    rng = np.random.default_rng(seed)
    locs = rng.uniform(0, 1, (n, 3))
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    w = rng.uniform(0.5, 1.0, n)
    return locs, nrm, w


def kernel_obj(name):
    from tbempy import ThreeD
    k = getattr(ThreeD, name)
    return k(1.0, 0.25) if name.startswith("Elastic") else k()


def make_pair(name, locs, nrm, w, order, leaf, small, precision="fp64", obs=None, m2l_path=0):
    from tbempy import ThreeD
    ol, on = (locs, nrm) if obs is None else obs
    orc = oracle.OracleFMM(name, ol, on, locs, nrm, w, 0.3, order, leaf, 0.05, small)
    op = ThreeD.FMMOperator(kernel_obj(name), ol, on, locs, nrm, w,
                            ThreeD.FMMConfig(0.3, order, leaf, 0.05, small), precision=precision,
                            m2l_path=m2l_path)
    return orc, op


def inject(op, orc):
    for which in (0, 1):
        assert op.n_c2e_levels(which) == len(orc.c2e[which])
        for lev in range(op.n_c2e_levels(which)):
            op.set_c2e(which, lev, orc.c2e[which][lev])


@pytest.mark.parametrize("name", KERNELS)
@pytest.mark.parametrize("small", [False, True])
def test_plain_matches_oracle(name, small):
    locs, nrm, w = cloud(800, 1)
    order = 35 if name.startswith("Laplace") else 20
    orc, op = make_pair(name, locs, nrm, w, order, 25, small)
    inject(op, orc)
    x = np.random.default_rng(2).uniform(-1, 1, op.n_cols())
    y = op.apply(x)
    y_orc = orc.apply(x)
    assert rel(y, y_orc) < 1e-10


@pytest.mark.parametrize("block", [1, 2, 4])
def test_p2m_variants_match_oracle(block):
    """Every threads-per-target variant of the points-to-check-surface pass
    (the autotuner's candidates) gives the reference's plain-form result."""
    from tbempy import ThreeD
    locs, nrm, w = cloud(800, 1)
    for name in ("LaplaceDouble", "ElasticTraction"):
        order = 35 if name.startswith("Laplace") else 20
        orc = oracle.OracleFMM(name, locs, nrm, locs, nrm, w, 0.3, order, 25, 0.05, False)
        op = ThreeD.FMMOperator(kernel_obj(name), locs, nrm, locs, nrm, w,
                                ThreeD.FMMConfig(0.3, order, 25, 0.05, False), p2m_block=block)
        inject(op, orc)
        x = np.random.default_rng(2).uniform(-1, 1, op.n_cols())
        assert rel(op.apply(x), orc.apply(x)) < 1e-10


@pytest.mark.parametrize("name", KERNELS)
def test_trees_and_lists_match_oracle(name):
    locs, nrm, w = cloud(700, 3)
    orc, op = make_pair(name, locs, nrm, w, 20, 15, True)
    for which in (0, 1):
        a, b = op.tree(which), orc.tree(which)
        for k in ("level", "index", "center", "hw", "n_idx", "n_children"):
            assert np.array_equal(a[k], b[k]), k
        for ia, ib in zip(a["indices"], b["indices"]):
            assert np.array_equal(ia, ib)
    for kind in oracle.LISTS:
        for u, v in zip(op.list(kind), orc.list(kind)):
            assert np.array_equal(u, v), kind


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES_3D = [p for p in sorted(glob.glob(os.path.join(GOLDEN, "fmm_*.npz")))
               if np.load(p)["src_locs"].shape[1] == 3]


@pytest.mark.parametrize("path", FIXTURES_3D, ids=[os.path.basename(p)[4:-4] for p in FIXTURES_3D])
def test_plain_own_operators_within_reference_floor(path):
    """The plain form with its OWN check-to-equivalent operators (cuSOLVER,
    one factorisation per tree side scaled per level) against the reference's
    apply on the reference's fixture.  The bar is the reference's own
    conditioning floor -- how far its result moves when every
    check-to-equivalent system is perturbed by one ulp before its
    pseudo-inverse (measured on the CPU, or stored with the fixture) -- at
    max(1e-10, 10 floors) (measured on GB300: 0.6 to 1.5 floors)."""
    from tbempy import ThreeD
    g = dict(np.load(path))
    cfg = ThreeD.FMMConfig(float(g["mac"]), int(g["order"]), int(g["leaf"]), float(g["d"]),
                           bool(g["small"]))
    op = ThreeD.FMMOperator(kernel_obj(str(g["kernel"])), g["obs_locs"], g["obs_normals"],
                            g["src_locs"], g["src_normals"], g["src_weights"], cfg)
    y = op.apply(g["x"])
    if "ulp_floor" in g:
        floor = float(g["ulp_floor"])
    else:
        orc = oracle.OracleFMM(str(g["kernel"]), g["obs_locs"], g["obs_normals"], g["src_locs"],
                               g["src_normals"], g["src_weights"], float(g["mac"]),
                               int(g["order"]), int(g["leaf"]), float(g["d"]), bool(g["small"]))
        floor = orc.ulp_floor(g["x"])
    err = rel(y, g["y_ref"])
    print("own operators: %.3g of the reference's apply, floor %.3g" % (err, floor))
    assert err <= max(1e-10, 10 * floor), "%.3g vs floor %.3g" % (err, floor)


def test_distinct_trees_plain():
    locs, nrm, w = cloud(700, 6)
    ol, on, _ = cloud(400, 7)
    for name in ("LaplaceSingle", "ElasticTraction"):
        order = 35 if name.startswith("Laplace") else 20
        orc, op = make_pair(name, locs, nrm, w, order, 25, False, obs=(ol, on))
        inject(op, orc)
        x = np.random.default_rng(8).uniform(-1, 1, op.n_cols())
        assert rel(op.apply(x), orc.apply(x)) < 1e-10


@pytest.mark.parametrize("name", KERNELS)
def test_mixed_vs_direct(name):
    """Precision form at the workload orders (152 / 296 requested surface
    points) against the FP64 direct sum: <= 2e-6 relative L2."""
    from tbempy import ThreeD, meshes
    locs, nrm, w = meshes.sphere_points(3)  # 3,840 points
    order = 152 if name.startswith("Laplace") else 296
    op = ThreeD.FMMOperator(kernel_obj(name), locs, nrm, locs, nrm, w,
                            ThreeD.FMMConfig(0.3, order, 40, 0.05, False), precision="mixed")
    x = np.random.default_rng(9).uniform(-1, 1, op.n_cols())
    exact = ThreeD.DirectOperator(kernel_obj(name), locs, nrm, locs, nrm, w).apply(x)
    err = rel(op.apply(x), exact)
    assert err < 2e-6, err


@pytest.mark.parametrize("name", ["LaplaceDouble", "ElasticDisplacement", "ElasticTraction"])
def test_mixed_distinct_points_compressed(name):
    """Different observation and source points (observers on a plane above a
    bumpy fault): both trees come from one cube, so the M2L between them is
    precomputed and compressed (nonzero ranks) and runs on the tensor cores;
    forward against the FP64 direct sum at 2e-6, and the transposed apply
    against the forward one, <A x, z> = <x, A^T z>, at 1e-6."""
    from tbempy import ThreeD, meshes
    v, t, obs, on, _, _, _ = meshes.misfit_workload(n=24, n_obs=3000)
    sl, sn, sw = meshes.points_from_mesh(v, t)
    K = kernel_obj(name)
    op = ThreeD.FMMOperator(K, obs, on, sl, sn, sw, ThreeD.FMMConfig(0.3, 296, 64, 0.05, False),
                            precision="mixed")
    assert op.m2l_ranks()[0] > 0 and op.tc_tile() > 0
    rng = np.random.default_rng(12)
    x = rng.uniform(-1, 1, op.n_cols())
    y = op.apply(x)
    exact = ThreeD.DirectOperator(K, obs, on, sl, sn, sw).apply(x)
    assert rel(y, exact) < 2e-6
    z = rng.uniform(-1, 1, op.n_rows())
    assert abs(y @ z - x @ op.apply_adjoint(z)) <= 1e-6 * np.linalg.norm(y) * np.linalg.norm(z)


@pytest.mark.parametrize("name,order", [("LaplaceSingle", 152), ("ElasticTraction", 296)])
def test_mixed_tensor_core_m2l_matches_simt(name, order):
    """tcgen05 3xBF16 M2L against the FP32 SIMT M2L on the same operators."""
    from tbempy import ThreeD, meshes
    locs, nrm, w = meshes.sphere_points(3)
    cfg = ThreeD.FMMConfig(0.3, order, 40, 0.05, False)
    tc = ThreeD.FMMOperator(kernel_obj(name), locs, nrm, locs, nrm, w, cfg, precision="mixed",
                            m2l_path=2)
    simt = ThreeD.FMMOperator(kernel_obj(name), locs, nrm, locs, nrm, w, cfg, precision="mixed",
                              m2l_path=1)
    X = np.random.default_rng(22).uniform(-1, 1, (3, tc.n_cols()))
    assert rel(tc.apply(X), simt.apply(X)) < 2e-6
    assert tc.tc_tile() in (64, 128) and simt.tc_tile() == 0
    assert tc.p2p_block() in (2, 4, 8)
    # M2M and L2L on the tensor cores as well
    full = ThreeD.FMMOperator(kernel_obj(name), locs, nrm, locs, nrm, w, cfg, precision="mixed",
                              m2l_path=3)
    assert rel(full.apply(X), simt.apply(X)) < 2e-6


@pytest.mark.parametrize("name,order", [("LaplaceSingle", 296), ("ElasticTraction", 296)])
def test_compressed_m2l(name, order):
    """SVD-compressed M2L (the default path of the precision form) against
    the uncompressed FP32 M2L on the same operators, and its transposed
    apply against the forward one through <A x, z> = <x, A^T z>."""
    from tbempy import ThreeD, meshes
    locs, nrm, w = meshes.sphere_points(3)
    cfg = ThreeD.FMMConfig(0.3, order, 40, 0.05, False)
    K = kernel_obj(name)
    comp = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed")
    simt = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed", m2l_path=1)
    n = comp.n_surface() * K.tensor_dim
    ri, ro = comp.m2l_ranks()
    assert 0 < ri <= n and 0 < ro <= n and ri * ro <= n * n // 2, (ri, ro, n)
    assert ri % 16 == 0 or ri == n
    assert simt.m2l_ranks() == (0, 0)
    rng = np.random.default_rng(31)
    X = rng.uniform(-1, 1, (3, comp.n_cols()))
    assert rel(comp.apply(X), simt.apply(X)) < 1e-6
    # a looser cut keeps fewer vectors and still approximates
    loose = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed",
                               m2l_rank_tol=1e-4)
    li, lo = loose.m2l_ranks()
    assert li <= ri and lo <= ro and li * lo < ri * ro
    assert rel(loose.apply(X), simt.apply(X)) < 1e-3
    # the M2L products on the tensor cores (3xBF16 split)
    tcc = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed", m2l_path=5)
    assert tcc.m2l_ranks() == (ri, ro) and tcc.tc_tile() in (64, 128)
    assert rel(tcc.apply(X), comp.apply(X)) < 2e-6
    Z = rng.uniform(-1, 1, (3, comp.n_rows()))
    AX = comp.apply(X)
    AtZ = comp.apply_adjoint(Z)
    for r in range(3):
        lhs, rhs = AX[r] @ Z[r], X[r] @ AtZ[r]
        assert abs(lhs - rhs) <= 1e-6 * np.linalg.norm(AX[r]) * np.linalg.norm(Z[r])


@pytest.mark.parametrize("shape", [1, 2, 3, 4])
def test_tensor_core_tile_shapes(shape):
    """Every tile shape the tensor-core autotuner can pick (N 128 / 64 columns,
    64- or 32-deep K chunks with 128- or 64-byte swizzle) against the FP32
    SIMT products on the same compressed operators."""
    from tbempy import ThreeD, meshes
    locs, nrm, w = meshes.sphere_points(3)
    cfg = ThreeD.FMMConfig(0.3, 296, 40, 0.05, False)
    K = kernel_obj("ElasticTraction")
    tcs = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed", m2l_path=5,
                             tc_shape=shape)
    simt = ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision="mixed", m2l_path=4)
    assert tcs.tc_tile() == {1: 128, 2: 64, 3: 128, 4: 256}[shape]
    X = np.random.default_rng(40).uniform(-1, 1, (2, tcs.n_cols()))
    assert rel(tcs.apply(X), simt.apply(X)) < 2e-6


@pytest.mark.parametrize("name", ["LaplaceDouble", "ElasticDisplacement"])
def test_plain_form_is_deterministic(name):
    """The plain form accumulates in conflict-free waves (no float atomics):
    repeated applies agree bit for bit, so FP64 residuals are reproducible."""
    locs, nrm, w = cloud(1200, 23)
    ol, on, _ = cloud(500, 24)
    for obs in (None, (ol, on)):
        orc, op = make_pair(name, locs, nrm, w, 35, 25, False, obs=obs)
        x = np.random.default_rng(25).uniform(-1, 1, op.n_cols())
        y0 = op.apply(x)
        for _ in range(3):
            assert np.array_equal(op.apply(x), y0)
        z = np.random.default_rng(26).uniform(-1, 1, op.n_rows())
        w0 = op.apply_adjoint(z)
        assert np.array_equal(op.apply_adjoint(z), w0)


def test_multi_rhs_matches_single():
    locs, nrm, w = cloud(900, 10)
    for prec in ("fp64", "mixed"):
        orc, op = make_pair("ElasticDisplacement", locs, nrm, w, 20, 30, False, precision=prec)
        X = np.random.default_rng(11).uniform(-1, 1, (6, op.n_cols()))
        Y = op.apply(X)
        for r in range(6):
            assert rel(Y[r], op.apply(X[r])) < (1e-12 if prec == "fp64" else 1e-6)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["LaplaceDouble", "ElasticTraction"])
def test_adjoint_is_transpose(prec, name):
    locs, nrm, w = cloud(300, 12)
    ol, on, _ = cloud(250, 13)
    for obs in (None, (ol, on)):
        # the transposed passes run on the FP32 pipes: compare with the same pipes forward
        orc, op = make_pair(name, locs, nrm, w, 20, 20, True, precision=prec, obs=obs, m2l_path=1)
        nc, nr = op.n_cols(), op.n_rows()
        A = op.apply(np.eye(nc)).T           # column j = A e_j
        At = op.apply_adjoint(np.eye(nr)).T  # column i = A^T e_i
        tol = 1e-12 if prec == "fp64" else 1e-6
        assert np.linalg.norm(A.T - At) / np.linalg.norm(A) < tol


@pytest.mark.parametrize("name", KERNELS)
def test_direct_matches_oracle(name):
    from tbempy import ThreeD
    locs, nrm, w = cloud(500, 14)
    ol, on, _ = cloud(300, 15)
    R = 3 if name.startswith("Elastic") else 1
    x = np.random.default_rng(16).uniform(-1, 1, R * len(locs))
    op = ThreeD.DirectOperator(kernel_obj(name), ol, on, locs, nrm, w)
    assert rel(op.apply(x), oracle.direct(name, ol, on, locs, nrm, w, x)) < 1e-13


def test_csr_apply():
    from tbempy import ThreeD
    rng = np.random.default_rng(17)
    n_rows, n_cols, nnz = 300, 200, 2500
    rows = rng.integers(0, n_rows, nnz)
    cols = rng.integers(0, n_cols, nnz)
    vals = rng.normal(size=nnz)
    op = ThreeD.SparseOperator.csr_from_coo(n_rows, n_cols, rows, cols, vals)
    dense = np.zeros((n_rows, n_cols))
    np.add.at(dense, (rows, cols), vals)
    X = rng.normal(size=(3, n_cols))
    assert rel(op.apply(X), X @ dense.T) < 1e-14
    assert op.nnz() == nnz


def test_empty_operators():
    from tbempy import ThreeD
    locs, nrm, w = cloud(50, 18)
    e3 = np.zeros((0, 3))
    cfg = ThreeD.FMMConfig(0.3, 20, 10, 0.05, False)
    op = ThreeD.FMMOperator(ThreeD.LaplaceSingle(), e3, e3, locs, nrm, w, cfg)
    assert op.n_rows() == 0 and op.apply(np.ones(50)).shape == (0,)
    op = ThreeD.FMMOperator(ThreeD.LaplaceSingle(), locs, nrm, e3, e3, np.zeros(0), cfg)
    assert np.all(op.apply(np.zeros(0)) == 0) and op.n_rows() == 50


def test_identity_kernel_known_answer():
    """Identity kernel: every output equals sum_j w_j x_j (cf. the reference's
    IdentityOperations known answers, unit_tests/test_fmm.cpp:31-68)."""
    from tbempy import ThreeD
    locs, nrm, _ = cloud(500, 19)
    w = np.ones(500)
    cfg = ThreeD.FMMConfig(0.3, 6, 8, 0.05, False)
    op = ThreeD.FMMOperator(ThreeD.IdentityScalar(), locs, nrm, locs, nrm, w, cfg)
    y = op.apply(np.ones(500))
    # the reference zeroes the self pair (r^2 < 1e-12), so each point sees n - 1
    assert np.allclose(y, 499.0, rtol=1e-9)


def test_torch_device_tensors():
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD
    locs, nrm, w = cloud(600, 20)
    op = ThreeD.FMMOperator(ThreeD.LaplaceSingle(), locs, nrm, locs, nrm, w,
                            ThreeD.FMMConfig(0.3, 35, 25, 0.05, False))
    x = np.random.default_rng(21).uniform(-1, 1, 600)
    y_np = op.apply(x)
    y_t = op.apply(torch.tensor(x, device="cuda"))
    assert y_t.is_cuda and rel(y_t.cpu().numpy(), y_np) < 1e-12  # float atomics order


def test_phase_timing_means_over_applies():
    """tbem_fmm_phase_times: mean device ms per apply of every phase over the
    applies since the previous read; no apply synchronizes for it."""
    torch = pytest.importorskip("torch")
    from tbempy import ThreeD, meshes
    locs, nrm, w = meshes.sphere_points(3)
    op = ThreeD.FMMOperator(ThreeD.ElasticDisplacement(1.0, 0.25), locs, nrm, locs, nrm, w,
                            ThreeD.FMMConfig(0.3, 296, 40, 0.05, False), precision="mixed")
    x = torch.rand(op.n_cols(), dtype=torch.float64, device="cuda")
    op.set_timing(True)
    for _ in range(3):
        op.apply(x)
    ph = dict(op.phase_times())
    # the compressed form runs the near field on a second stream: its phase is
    # the wait for it after the far field
    assert {"gather", "p2m", "m2m", "m2l", "l2l", "p2p_wait", "l2p", "scatter"} <= set(ph)
    assert all(t >= 0 for t in ph.values()) and ph["m2l"] > 0
    assert dict(op.phase_times()) == ph  # nothing new: the same numbers
    op.set_timing(False)
    op.apply(x)
    assert dict(op.phase_times()) == ph
    # the FMA-rate microbenchmark (the evaluation kernels' denominator): FP32
    # well above FP64, both within a plausible range for one GPU
    f32, f64 = ThreeD.fma_peak_tflops(False), ThreeD.fma_peak_tflops(True)
    assert 10.0 < f32 < 400.0 and 0.05 < f64 < f32
    # construction phases, in order
    names = [n for n, _ in op.setup_times()]
    assert names == ["trees_lists", "upload_tasks", "c2e", "translations", "compression",
                     "leaf_operators", "autotune"]
    assert all(s >= 0 for _, s in op.setup_times())


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_compressed"])
def test_setup_cache_reuse_matches_a_fresh_build(precision):
    """A traction operator built after another operator with the same
    translation kernel over the same points (the precision forms translate
    with the displacement kernel whatever the operator's kernel; the plain
    form with the operator's own) takes its pseudo-inverses and M2L
    eigenbases from the setup cache: they are bit-identical to those of a
    build from an empty cache, and so are the ranks; the two applies agree
    to the form's summation-order noise."""
    from tbempy import ThreeD
    locs, nrm, w = cloud(3000, 41)
    cfg = ThreeD.FMMConfig(0.3, 152 if precision == "fp64" else 296, 40, 0.05, False)

    def build(K):
        return ThreeD.FMMOperator(K, locs, nrm, locs, nrm, w, cfg, precision=precision)

    ThreeD.clear_setup_cache()
    first = ThreeD.ElasticTraction(1.0, 0.25) if precision == "fp64" else \
        ThreeD.ElasticDisplacement(1.0, 0.25)
    t0 = dict(build(first).setup_times())
    warm = build(ThreeD.ElasticTraction(1.0, 0.25))
    ThreeD.clear_setup_cache()
    cold = build(ThreeD.ElasticTraction(1.0, 0.25))
    for which in (0, 1):
        assert warm.n_c2e_levels(which) == cold.n_c2e_levels(which)
        for lev in range(cold.n_c2e_levels(which)):
            assert np.array_equal(warm.get_c2e(which, lev), cold.get_c2e(which, lev))
    assert warm.m2l_ranks() == cold.m2l_ranks()
    x = np.random.default_rng(42).uniform(-1, 1, cold.n_cols())
    yw, yc = warm.apply(x), cold.apply(x)
    assert rel(yw, yc) < {"fp64": 1e-12, "fp64_compressed": 1e-10, "mixed": 1e-6}[precision]
    # the reused phase takes a fraction of the factoring one
    assert dict(warm.setup_times())["c2e"] < 0.5 * t0["c2e"] + 0.01


@pytest.mark.parametrize("name", KERNELS)
def test_default_precision_form_transpose(name):
    """The default precision form (compressed far field, tensor-core M2L) and
    its transposed apply: <A x, z> = <x, A^T z> for every kernel."""
    from tbempy import ThreeD, meshes
    locs, nrm, w = meshes.sphere_points(3)
    order = 152 if name.startswith("Laplace") else 296
    op = ThreeD.FMMOperator(kernel_obj(name), locs, nrm, locs, nrm, w,
                            ThreeD.FMMConfig(0.3, order, 40, 0.05, False), precision="mixed")
    rng = np.random.default_rng(60)
    X = rng.uniform(-1, 1, (2, op.n_cols()))
    Z = rng.uniform(-1, 1, (2, op.n_rows()))
    AX, AtZ = op.apply(X), op.apply_adjoint(Z)
    for r in range(2):
        lhs, rhs = AX[r] @ Z[r], X[r] @ AtZ[r]
        assert abs(lhs - rhs) <= 1e-6 * np.linalg.norm(AX[r]) * np.linalg.norm(Z[r])


@pytest.mark.parametrize("prec", ["mixed", "fp64_compressed"])
@pytest.mark.parametrize("name", ["LaplaceSingle", "ElasticDisplacement"])
@pytest.mark.parametrize("distinct", [False, True])
def test_compressed_adjoint_many_rhs(name, distinct, prec):
    """The compressed forms' transposed apply: 1 to 64 right-hand sides at
    once equal the same right-hand sides one at a time, whatever forward
    applies left in the work buffers, and equal the transpose of the forward
    operator (every leaf's transposed P2M reads only states of this apply)."""
    from tbempy import ThreeD
    src, sn, w = cloud(400, 1)
    ol, on = (src, sn) if not distinct else cloud(300, 2)[:2]
    op = ThreeD.FMMOperator(kernel_obj(name), ol, on, src, sn, w,
                            ThreeD.FMMConfig(0.3, 296, 30, 0.05, False), precision=prec)
    rng = np.random.default_rng(5)
    Z = rng.uniform(-1, 1, (64, op.n_rows()))
    X = rng.uniform(-1, 1, (64, op.n_cols()))
    tol = 1e-6 if prec == "mixed" else 1e-12
    single = []
    for i in range(16):
        op.apply(X[i])  # leaves forward states behind
        single.append(op.apply_adjoint(Z[i]))
    single = np.stack(single)
    for nr in (2, 3, 5, 16):
        op.apply(X[:nr])
        W = op.apply_adjoint(Z[:nr])
        assert np.all(np.isfinite(W))
        assert rel(W, single[:nr]) < tol
    AX = op.apply(X[:16])
    W = op.apply_adjoint(Z[:16])
    for r in range(16):
        lhs, rhs = AX[r] @ Z[r], X[r] @ W[r]
        assert abs(lhs - rhs) <= 10 * tol * np.linalg.norm(AX[r]) * np.linalg.norm(Z[r])


@pytest.mark.parametrize("name", ["LaplaceDouble", "ElasticTraction"])
def test_precision_form_distinct_point_sets(name):
    """Observation points apart from the sources (a free surface above the
    fault): both trees come from one cube, so the precision form's M2L
    between them is precomputed and compressed; against the FP64 direct sum."""
    from tbempy import ThreeD, meshes
    locs, nrm, w, uv = meshes.fault_points(16)
    rng = np.random.default_rng(61)
    obs = np.column_stack([rng.uniform(-2, 2, 3000), rng.uniform(-2, 2, 3000), np.zeros(3000)])
    on = np.tile([0.0, 0.0, 1.0], (3000, 1))
    K = kernel_obj(name)
    order = 152 if name.startswith("Laplace") else 296
    op = ThreeD.FMMOperator(K, obs, on, locs, nrm, w, ThreeD.FMMConfig(0.3, order, 40, 0.05, False),
                            precision="mixed")
    assert op.m2l_ranks()[0] > 0  # compressed between the two trees
    x = rng.uniform(-1, 1, op.n_cols())
    exact = ThreeD.DirectOperator(K, obs, on, locs, nrm, w).apply(x)
    assert rel(op.apply(x), exact) < 2e-6
