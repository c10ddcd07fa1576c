"""GPU parity of the 2D operators (the reference's FMMOperator<2,1,1> and
<2,2,2>: quadtrees, circle surfaces, the 2D Laplace and elastic kernels) and
of every golden fixture, 3D and 2D, against the reference's own outputs.

Tolerances (written here, checked below):
  * plain FP64 FMM with the reference's own check-to-equivalent operators
    installed vs the reference's apply (fixtures) or the oracle: 1e-10
    relative L2, or -- for the 2D operators -- 100 x the case's conditioning
    floor when that is larger (10 x the floor stored with a 3D fixture at a
    high order: the 152-point icosphere case, floor 2.7e-8).  The floor is
    measured on the CPU: the
    relative change of the oracle's own apply when its check-to-equivalent
    systems are perturbed by one ulp (OracleFMM.ulp_floor).  The reference
    algorithm keeps singular values down to 1e-10 of the largest, and with
    the 2D kernels of the 1/r and log families that moves the result by up
    to ~3e-8 for a one-ulp change in its inputs (3D kernels, 2D
    hypersingular kernels: <= 1e-11), so no two correct FP64 evaluations
    agree closer than that (measured on GB300: the GPU lands within 0.8 to
    5 floors of the reference and the oracle, and within 1e-10 wherever the
    floor is below 1e-12);
  * GPU FP64 direct sum vs the reference's nbody_eval (fixtures) and vs the
    oracle: 1e-12 relative L2 (summation order only);
  * transposed apply vs the dense transpose of the forward apply, and a
    multi-RHS apply vs single applies: 1e-12, or 100 x the floor (2D);
  * the reference's own 2D FMM accuracy cases (unit_tests/test_fmm.cpp:109-149)
    with the GPU's cuSOLVER pseudo-inverses: the reference's bounds (1e-4,
    1e-2 for the order-5 single layer) in its min(relative, mean-scaled)
    error measure.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "fmm_*.npz")))
KERNELS_2D = ["LaplaceSingle", "LaplaceDouble", "LaplaceHypersingular", "ElasticDisplacement",
              "ElasticTraction", "ElasticAdjointTraction", "ElasticHypersingular"]


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def kernel_obj(name, dim, mu=1.0, nu=0.25):
    from tbempy import ThreeD, TwoD
    k = getattr(TwoD if dim == 2 else ThreeD, name)
    return k(mu, nu) if name.startswith("Elastic") else k()


def tol_2d(orc, x):
    """max(1e-10, 100 x the conditioning floor of this case)."""
    return max(1e-10, 100 * orc.ulp_floor(x))


def cloud2(n, seed, lo=0.0, hi=1.0):
    rng = np.random.default_rng(seed)
    locs = rng.uniform(lo, hi, (n, 2))
    nrm = rng.normal(size=(n, 2))
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    return locs, nrm, rng.uniform(0.5, 1.0, n)


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[4:-4] for p in CASES])
def test_plain_form_reproduces_reference_fixture(path):
    from tbempy import ThreeD
    g = dict(np.load(path))
    dim = g["src_locs"].shape[1]
    K = kernel_obj(str(g["kernel"]), dim)
    cfg = ThreeD.FMMConfig(float(g["mac"]), int(g["order"]), int(g["leaf"]), float(g["d"]),
                           bool(g["small"]))
    op = ThreeD.FMMOperator(K, g["obs_locs"], g["obs_normals"], g["src_locs"], g["src_normals"],
                            g["src_weights"], cfg)
    for which in (0, 1):
        ops = g["c2e%d" % which]
        assert op.n_c2e_levels(which) == len(ops)
        for lev, m in enumerate(ops):
            op.set_c2e(which, lev, m)
    tol = 1e-10
    if "ulp_floor" in g:
        # 3D at a high order (the 15,360-point icosphere at 152 surface
        # points): the reference's own one-ulp floor is above 1e-10 (2.7e-8),
        # so two correct FP64 evaluations of its algorithm -- even with the
        # same pseudo-inverses -- differ by a fraction of that floor (measured
        # on GB300: 0.35 floors); the bar is 10 floors there
        tol = max(1e-10, 10 * float(g["ulp_floor"]))
    if dim == 2:
        orc = oracle.OracleFMM(str(g["kernel"]), g["obs_locs"], g["obs_normals"], g["src_locs"],
                               g["src_normals"], g["src_weights"], float(g["mac"]),
                               int(g["order"]), int(g["leaf"]), float(g["d"]), bool(g["small"]))
        tol = tol_2d(orc, g["x"])
    assert rel(op.apply(g["x"]), g["y_ref"]) < tol
    d = ThreeD.DirectOperator(K, g["obs_locs"], g["obs_normals"], g["src_locs"], g["src_normals"],
                              g["src_weights"])
    assert rel(d.apply(g["x"]), g["y_direct"]) < 1e-12


@pytest.mark.parametrize("name", KERNELS_2D + ["IdentityScalar"])
def test_2d_direct_matches_oracle(name):
    from tbempy import TwoD
    locs, nrm, w = cloud2(500, 21)
    ol, on, _ = cloud2(300, 22, -0.5, 1.5)
    K = kernel_obj(name, 2, 1.7, 0.3)
    x = np.random.default_rng(23).uniform(-1, 1, K.tensor_dim * len(locs))
    y = TwoD.DirectOperator(K, ol, on, locs, nrm, w).apply(x)
    assert rel(y, oracle.direct(K.kernel_id, ol, on, locs, nrm, w, x, mu=1.7, nu=0.3)) < 1e-12


@pytest.mark.parametrize("name", KERNELS_2D)
@pytest.mark.parametrize("small", [False, True])
def test_2d_plain_matches_oracle(name, small):
    """Distinct observation and source sets, multi-RHS, reference operators
    (the oracle's LAPACK pseudo-inverses) installed: 1e-10 or 100 floors."""
    from tbempy import ThreeD, TwoD
    locs, nrm, w = cloud2(900, 24, -1, 1)
    ol, on, _ = cloud2(600, 25, -0.8, 1.3)
    K = kernel_obj(name, 2, 1.3, 0.27)
    orc = oracle.OracleFMM(K.kernel_id, ol, on, locs, nrm, w, 0.3, 20, 15, 0.05, small,
                           mu=1.3, nu=0.27)
    op = TwoD.FMMOperator(K, ol, on, locs, nrm, w, ThreeD.FMMConfig(0.3, 20, 15, 0.05, small))
    for which in (0, 1):
        for lev in range(op.n_c2e_levels(which)):
            op.set_c2e(which, lev, orc.c2e[which][lev])
    X = np.random.default_rng(26).uniform(-1, 1, (3, op.n_cols()))
    Y = op.apply(X)
    floor = orc.ulp_floor(X[0])
    for r in range(3):
        assert rel(Y[r], orc.apply(X[r])) < max(1e-10, 100 * floor)
        assert rel(op.apply(X[r]), Y[r]) < max(1e-12, 100 * floor)


@pytest.mark.parametrize("name", ["LaplaceDouble", "LaplaceHypersingular", "ElasticTraction",
                                  "ElasticHypersingular"])
def test_2d_adjoint_is_transpose(name):
    from tbempy import ThreeD, TwoD
    locs, nrm, w = cloud2(260, 27)
    ol, on, _ = cloud2(200, 28, 0.2, 1.4)
    K = kernel_obj(name, 2)
    op = TwoD.FMMOperator(K, ol, on, locs, nrm, w, ThreeD.FMMConfig(0.3, 16, 12, 0.05, True))
    orc = oracle.OracleFMM(K.kernel_id, ol, on, locs, nrm, w, 0.3, 16, 12, 0.05, True)
    nc, nr = op.n_cols(), op.n_rows()
    floor = orc.ulp_floor(np.random.default_rng(30).uniform(-1, 1, nc))
    A = op.apply(np.eye(nc)).T
    At = op.apply_adjoint(np.eye(nr)).T
    assert np.linalg.norm(A.T - At) / np.linalg.norm(A) < max(1e-12, 100 * floor)


@pytest.mark.parametrize("name,order,tol,mu", [
    ("IdentityScalar", 1, 1e-4, 1.0), ("LaplaceSingle", 5, 1e-2, 1.0),
    ("LaplaceDouble", 20, 1e-4, 1.0), ("LaplaceHypersingular", 20, 1e-4, 1.0),
    ("ElasticDisplacement", 20, 1e-4, 30e9), ("ElasticTraction", 20, 1e-4, 30e9),
    ("ElasticHypersingular", 30, 1e-4, 30e9)])
def test_2d_reference_accuracy_cases(name, order, tol, mu):
    """unit_tests/test_fmm.cpp:109-149 on the GPU with its own pseudo-inverses."""
    from tbempy import ThreeD, TwoD
    rng = np.random.default_rng(4)
    src, obs, nrm = rng.uniform(0, 1, (100, 2)), rng.uniform(0, 1, (100, 2)), rng.uniform(0, 1, (100, 2))
    K = kernel_obj(name, 2, mu, 0.25)
    op = TwoD.FMMOperator(K, obs, nrm, src, nrm, np.ones(100), ThreeD.FMMConfig(0.35, order, 1, 0.05, False))
    x = np.ones(op.n_cols())
    exact = TwoD.DirectOperator(K, obs, nrm, src, nrm, np.ones(100)).apply(x)
    avg = np.mean(np.abs(exact))
    d = op.apply(x) - exact
    with np.errstate(divide="ignore", invalid="ignore"):
        e1 = np.nan_to_num(np.abs(d / exact), nan=np.inf)
    assert np.all(np.minimum(e1, np.abs(d / avg)) <= tol)


def test_2d_clone_and_circle_boundary():
    """A clone (points narrowed back to [n][2]) applies the same operator; on
    a circle the single layer of a constant density is the known constant
    log(1) = 0 inside up to the discretisation error."""
    from tbempy import ThreeD, TwoD
    n = 2048
    t = 2 * np.pi * (np.arange(n) + 0.5) / n
    pts = np.stack([np.cos(t), np.sin(t)], axis=1)
    w = np.full(n, 2 * np.pi / n)
    op = TwoD.FMMOperator(TwoD.LaplaceSingle(), pts, pts, pts, pts, w,
                          ThreeD.FMMConfig(0.3, 24, 32, 0.05, False))
    x = np.random.default_rng(29).uniform(-1, 1, n)
    c = op.clone()
    assert np.array_equal(c.apply(x), op.apply(x))
    inner = 0.5 * pts[:64]
    d = TwoD.DirectOperator(TwoD.LaplaceSingle(), inner, inner, pts, pts, w).apply(np.ones(n))
    assert np.abs(d).max() < 1e-10
