"""CPU tests: the oracle (restatement of the reference KIFMM) pinned against
the reference's own outputs (golden fixtures made by tests/golden/make_golden.py
from the reference compiled from its sources), against the reference's
known-answer tests, and -- where the reference checkout is present -- against
the reference library itself."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(glob.glob(os.path.join(GOLDEN, "fmm_*.npz")))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def load(path):
    return dict(np.load(path, allow_pickle=False))


def oracle_for(g):
    return oracle.OracleFMM(str(g["kernel"]), g["obs_locs"], g["obs_normals"], g["src_locs"],
                            g["src_normals"], g["src_weights"], float(g["mac"]), int(g["order"]),
                            int(g["leaf"]), float(g["d"]), bool(g["small"]))


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[4:-4] for p in CASES])
def test_oracle_matches_reference_fixture(path):
    g = load(path)
    o = oracle_for(g)
    assert o.n_surf() == int(g["n_surf"])
    for which in (0, 1):
        t = o.tree(which)
        for k in ("level", "index", "center", "hw", "n_idx", "n_children"):
            assert np.array_equal(t[k], g["tree%d_%s" % (which, k)]), k
        assert np.array_equal(np.concatenate(t["indices"]), g["tree%d_indices" % which])
    for kind in oracle.LISTS:
        a, b = o.list(kind)
        assert np.array_equal(a, g["list_%s_obs" % kind]) and np.array_equal(b, g["list_%s_src" % kind])
    # the reference's own check-to-equivalent operators: the apply agrees to
    # rounding.  The oracle's OpenMP passes add in a thread-dependent order;
    # where the fixture carries the reference's one-ulp floor (the
    # 15,360-point icosphere, where that floor is 2.7e-8) a hundredth of it
    # bounds what a different order of the same sums may move
    for which in (0, 1):
        for lev, op in enumerate(g["c2e%d" % which]):
            o.set_c2e(which, lev, op)
    tol = max(1e-12, 0.01 * float(g["ulp_floor"])) if "ulp_floor" in g else 1e-12
    assert rel(o.apply(g["x"]), g["y_ref"]) < tol


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[4:-4] for p in CASES])
def test_direct_matches_reference_fixture(path):
    g = load(path)
    y = oracle.direct(str(g["kernel"]), g["obs_locs"], g["obs_normals"], g["src_locs"],
                      g["src_normals"], g["src_weights"], g["x"])
    assert rel(y, g["y_direct"]) < 1e-13


def test_pinv_matches_reference_operators():
    """The oracle's LAPACK pseudo-inverse reproduces the reference's operators."""
    g = load(os.path.join(GOLDEN, "fmm_laps_cube.npz"))
    o = oracle_for(g)
    for which in (0, 1):
        for lev, op in enumerate(g["c2e%d" % which]):
            assert np.linalg.norm(o.c2e[which][lev] - op) <= 1e-10 * np.linalg.norm(op)


def test_kernel_golden_vectors():
    rows = np.load(os.path.join(GOLDEN, "kernels.npz"))["rows"]
    for r in rows:
        k, mu, nu = int(r[0]), r[1], r[2]
        K = oracle.kernel_tensor(k, r[3:6], r[6:9], r[9:12], r[12:15], mu, nu)
        ref = r[15:15 + K.size].reshape(K.shape)
        assert np.allclose(K, ref, rtol=1e-14, atol=0), (k, K, ref)


def test_kernel_golden_vectors_2d():
    """The 2D kernels (ids 16-23) against the reference's own tensors, bit for bit."""
    g = np.load(os.path.join(GOLDEN, "kernels_2d.npz"))
    rows = g["rows"]
    assert sorted(set(rows[:, 0].astype(int))) == list(range(16, 24))
    for r in rows:
        k, mu, nu = int(r[0]), r[1], r[2]
        K = oracle.kernel_tensor(k, r[3:5], r[6:8], r[9:11], r[12:14], mu, nu)
        assert K.shape == ((2, 2) if 19 <= k <= 22 else (1, 1))
        assert np.array_equal(K, r[15:15 + K.size].reshape(K.shape)), (k, K)


def test_circle_surface_known_values():
    """unit_tests/test_fmm.cpp:21-29 (order 4) and the reference's point counts."""
    g = np.load(os.path.join(GOLDEN, "kernels_2d.npz"))
    s = oracle.surface(4, 2)
    assert np.array_equal(s, g["surf4"])
    assert np.allclose(s[0, :2], [1, 0], atol=1e-12) and np.allclose(s[1, :2], [0, 1], atol=1e-12)
    assert np.allclose(s[3, :2], [0, -1], atol=1e-12)
    for o, c in zip(g["surf_orders"], g["surf_counts"]):
        assert len(oracle.surface(int(o), 2)) == c == o


REF_ELASTIC = os.path.join(oracle.REF_ROOT, "unit_tests", "test_data_elastic3")


@pytest.mark.skipif(not os.path.exists(REF_ELASTIC), reason="reference checkout absent")
def test_elastic_kernels_against_reference_sympy_data():
    """The reference's symbolic golden data (unit_tests/test_data_elastic3,
    checked by unit_tests/test_elastic_kernels.cpp:54-103 at 1e-8)."""
    ids = {"disp": 2, "trac": 3, "adj_trac": 4, "hyp": 6}
    n = 0
    with open(REF_ELASTIC) as f:
        for line in f:
            e = line.strip().split(",")
            if e[1] not in ids:
                continue
            k, j = int(e[2]), int(e[3])
            v = [float(t) for t in e[8:20]]
            K = oracle.kernel_tensor(ids[e[1]], v[3:6], v[0:3], v[9:12], v[6:9], float(e[4]), float(e[5]))
            exact = float(e[0])
            if exact != 0.0:
                err = abs(exact - K[k, j]) / ((abs(exact) + abs(K[k, j])) / 2)
                assert err < 1e-8
            else:
                assert K[k, j] == 0.0
            n += 1
    assert n == 360


REF_ELASTIC_2D = os.path.join(oracle.REF_ROOT, "unit_tests", "test_data_elastic2")


@pytest.mark.skipif(not os.path.exists(REF_ELASTIC_2D), reason="reference checkout absent")
def test_elastic_kernels_2d_against_reference_sympy_data():
    """unit_tests/test_data_elastic2 through unit_tests/test_elastic_kernels.cpp:54-119
    (2D: the first two of each coordinate triple, 1e-8)."""
    ids = {"disp": 19, "trac": 20, "adj_trac": 21, "hyp": 22}
    n = 0
    with open(REF_ELASTIC_2D) as f:
        for line in f:
            e = line.strip().split(",")
            if e[1] not in ids:
                continue
            k, j = int(e[2]), int(e[3])
            v = [float(t) for t in e[8:20]]
            K = oracle.kernel_tensor(ids[e[1]], v[3:5], v[0:2], v[9:11], v[6:8], float(e[4]),
                                     float(e[5]))
            exact = float(e[0])
            if exact != 0.0:
                assert abs(exact - K[k, j]) / ((abs(exact) + abs(K[k, j])) / 2) < 1e-8
            else:
                assert K[k, j] == 0.0
            n += 1
    assert n == 160


def test_laplace_nbody_known_values():
    """unit_tests/test_nbody_operator.cpp:27-41."""
    obs = np.array([[0, 0, 0], [0, 2, 0], [0, 0, -1.0]])
    src = np.array([[1, 0, 0], [0, 1, 0.0]])
    y = oracle.direct("LaplaceSingle", obs, np.zeros((3, 3)), src, np.zeros((2, 3)),
                      np.ones(2), np.array([4.0, 0.0]))
    assert np.allclose(y, [0.3183, 0.1424, 0.2251], atol=1e-3)


def test_pseudoinverse_known_answers():
    """unit_tests/test_blas_wrapper.cpp:32-66."""
    assert np.allclose(oracle.pinv_reference(np.array([[2, 1], [-1, 0.5]]), 1e-16),
                       [[0.25, -0.5], [0.5, 1.0]], atol=1e-14)
    m = np.array([[0.0238032718573239, 0.1524037864980028],
                  [0.1524037864980028, 0.9762067281426762]])
    assert np.allclose(oracle.pinv_reference(m, 1e-16),
                       [[97620.6728142285282956, -15240.3786497941800917],
                        [-15240.3786497941782727, 2380.3271857314393856]], atol=1e-4)
    assert np.allclose(oracle.pinv_reference(m, 1e-4),
                       [[0.0237935097924219, 0.1524053105511083],
                        [0.1524053105511085, 0.9762064902075779]], atol=1e-12)


def test_surface_point_counts():
    g = load(os.path.join(GOLDEN, "misc.npz"))
    for o, c in zip(g["surf_orders"], g["surf_counts"]):
        assert len(oracle.surface(int(o))) == c


def test_degenerate_line_octree():
    """The reference's degenerate-line octree test (unit_tests/test_octree.cpp:144-155),
    restated in 3D; the count comes from the reference itself."""
    g = load(os.path.join(GOLDEN, "misc.npz"))
    line = g["line_pts"]
    o = oracle.OracleFMM("LaplaceSingle", line, np.ones_like(line), line, np.ones_like(line),
                         np.ones(len(line)), 0.3, 6, 1, 0.05, False)
    t = o.tree(0)
    assert len(t["level"]) == int(g["line_n_cells"])
    assert np.array_equal(t["n_idx"], g["line_n_idx"])


def test_octree_structure():
    """Point conservation, unique indices, balance (unit_tests/test_octree.cpp:22-111,173-178)."""
    rng = np.random.default_rng(0)
    pts = rng.uniform(0, 1, (20000, 3))
    o = oracle.OracleFMM("LaplaceSingle", pts[:10], np.ones((10, 3)), pts, np.ones_like(pts),
                         np.ones(len(pts)), 0.3, 6, 100, 0.05, False)
    t = o.tree(0)
    assert len(np.unique(t["index"])) == len(t["index"])
    assert t["n_idx"][0] == len(pts)
    # children of the root hold about n/8 points each
    kids = np.where(t["level"] == 1)[0]
    assert len(kids) == 8
    assert np.all(np.abs(t["n_idx"][kids] - len(pts) / 8) < len(pts) / 16)
    # leaves partition the points
    leaves = np.where(t["n_children"] == 0)[0]
    allpts = np.sort(np.concatenate([t["indices"][i] for i in leaves]))
    assert np.array_equal(allpts, np.arange(len(pts)))


def _ref_error(out, exact):
    """Per-entry min(|d/exact|, |d/mean|exact||) of unit_tests/test_fmm.cpp:70-98."""
    avg = np.mean(np.abs(exact))
    d = out - exact
    with np.errstate(divide="ignore", invalid="ignore"):
        e1 = np.abs(d / exact)
    return np.minimum(np.nan_to_num(e1, nan=np.inf), np.abs(d / avg))


@pytest.mark.parametrize("name,order", [("LaplaceSingle", 35), ("LaplaceDouble", 75)])
def test_oracle_fmm_accuracy_reference_cases(name, order):
    """unit_tests/test_fmm.cpp:129-137: 100 random points, mac 0.35, one point
    per cell, d = 0.05, error <= 1e-4 against the direct operator."""
    rng = np.random.default_rng(1)
    src, obs, nrm = rng.uniform(0, 1, (100, 3)), rng.uniform(0, 1, (100, 3)), rng.uniform(0, 1, (100, 3))
    o = oracle.OracleFMM(name, obs, nrm, src, nrm, np.ones(100), 0.35, order, 1, 0.05, False)
    x = np.ones(100)
    exact = oracle.direct(name, obs, nrm, src, nrm, np.ones(100), x)
    assert np.all(_ref_error(o.apply(x), exact) <= 1e-4)


@pytest.mark.parametrize("name,order,tol,mu", [
    ("IdentityScalar", 1, 1e-4, 1.0), ("LaplaceSingle", 5, 1e-2, 1.0),
    ("LaplaceDouble", 20, 1e-4, 1.0), ("LaplaceHypersingular", 20, 1e-4, 1.0),
    ("ElasticDisplacement", 20, 1e-4, 30e9), ("ElasticTraction", 20, 1e-4, 30e9),
    ("ElasticHypersingular", 30, 1e-4, 30e9)])
def test_oracle_fmm_accuracy_reference_cases_2d(name, order, tol, mu):
    """unit_tests/test_fmm.cpp:109-149 (2D): 100 random points in the unit
    square, unit weights, mac 0.35, one point per cell, d = 0.05."""
    rng = np.random.default_rng(4)
    src, obs, nrm = rng.uniform(0, 1, (100, 2)), rng.uniform(0, 1, (100, 2)), rng.uniform(0, 1, (100, 2))
    o = oracle.OracleFMM(name, obs, nrm, src, nrm, np.ones(100), 0.35, order, 1, 0.05, False,
                         mu=mu, nu=0.25)
    x = np.ones(o.R * 100)
    exact = oracle.direct(name, obs, nrm, src, nrm, np.ones(100), x, mu=mu, nu=0.25)
    assert np.all(_ref_error(o.apply(x), exact) <= tol)


def test_quadtree_known_answers():
    """unit_tests/test_octree.cpp:16-20, 54-62, 102-111: child order (x is the
    high bit), the degenerate 2D line splits, and points are conserved."""
    # child index 1 = (x low, y high), 3 = (high, high): place one point per quadrant
    pts = np.array([[-1.0, -1.0], [-1.0, 1.0], [1.0, -1.0], [1.0, 1.0]])
    o = oracle.OracleFMM("LaplaceSingle", pts, pts, pts, pts, np.ones(4), 0.3, 4, 1, 0.05, False)
    t = o.tree(0)
    kids = np.where(t["level"] == 1)[0]
    assert [int(t["indices"][c][0]) for c in kids] == [0, 1, 2, 3]
    line = np.array([[float(i), 0.0] for i in range(100)])
    for leaf in (1, 26):
        o = oracle.OracleFMM("LaplaceSingle", line, line, line, line, np.ones(100), 0.3, 4, leaf,
                             0.05, False)
        t = o.tree(0)
        assert t["n_children"][0] > 0
        leaves = np.where(t["n_children"] == 0)[0]
        assert np.array_equal(np.sort(np.concatenate([t["indices"][i] for i in leaves])),
                              np.arange(100))
        # a quadtree: at most four children, z untouched
        assert t["n_children"].max() <= 4 and not t["center"][:, 2].any() and not t["hw"][:, 2].any()


def test_identity_fmm_known_answer():
    rng = np.random.default_rng(2)
    pts = rng.uniform(0, 1, (300, 3))
    o = oracle.OracleFMM("IdentityScalar", pts, pts, pts, pts, np.ones(300), 0.3, 6, 8, 0.05, False)
    assert np.allclose(o.apply(np.ones(300)), 299.0, rtol=1e-9)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference library not built here")
@pytest.mark.parametrize("small", [False, True])
def test_oracle_vs_reference_library(small):
    rng = np.random.default_rng(3)
    pts = rng.uniform(0, 1, (1500, 3))
    nrm = rng.normal(size=(1500, 3))
    w = rng.uniform(0.5, 1, 1500)
    for name, order in (("LaplaceDouble", 35), ("ElasticTraction", 20), ("ElasticHypersingular", 20)):
        a = oracle.OracleFMM(name, pts, nrm, pts, nrm, w, 0.3, order, 30, 0.05, small)
        b = oracle.RefFMM(name, pts, nrm, pts, nrm, w, 0.3, order, 30, 0.05, small)
        for which in (0, 1):
            for lev in range(b.n_levels(which)):
                a.set_c2e(which, lev, b.c2e(which, lev))
        x = rng.uniform(-1, 1, a.R * 1500)
        assert rel(a.apply(x), b.apply(x)) < 1e-12


@pytest.mark.skipif(not oracle.ref_available(), reason="reference library not built here")
@pytest.mark.parametrize("small", [False, True])
def test_oracle_vs_reference_library_2d(small):
    """Every 2D kernel: identical trees and lists, and with the reference's
    own pseudo-inverses installed, the same apply to rounding (bit for bit
    with one thread; both sides scatter with OpenMP atomics otherwise)."""
    rng = np.random.default_rng(6)
    pts = rng.uniform(-1, 1, (800, 2))
    obs = rng.uniform(-1, 1, (700, 2)) + np.array([0.4, 0.1])
    nrm = rng.normal(size=(800, 2))
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    w = rng.uniform(0.5, 1.5, 800)
    for k in range(16, 24):
        a = oracle.OracleFMM(k, obs, nrm[:700], pts, nrm, w, 0.3, 16, 12, 0.05, small, mu=1.3, nu=0.27)
        b = oracle.RefFMM(k, obs, nrm[:700], pts, nrm, w, 0.3, 16, 12, 0.05, small, mu=1.3, nu=0.27)
        for which in (0, 1):
            ta, tb = a.tree(which), b.tree(which)
            for key in ("level", "index", "center", "hw", "n_idx", "n_children"):
                assert np.array_equal(ta[key], tb[key]), (k, key)
        for kind in oracle.LISTS:
            assert all(np.array_equal(u, v) for u, v in zip(a.list(kind), b.list(kind))), (k, kind)
        for which in (0, 1):
            for lev in range(b.n_levels(which)):
                a.set_c2e(which, lev, b.c2e(which, lev))
        x = rng.uniform(-1, 1, a.R * 800)
        assert rel(a.apply(x), b.apply(x)) < 1e-13, k


def test_hypersingular_is_the_traction_of_the_dislocation_field():
    """The precision form evaluates the hypersingular kernel as traction
    (observation normal) of the displacement field of its sources, carried by
    point-force equivalents: this holds in the reference's conventions, as it
    does for the adjoint traction and the displacement kernel (central
    differences of the field, sigma = lambda tr(grad u) I + mu (grad u +
    grad u^T))."""
    rng = np.random.default_rng(7)
    mu, nu = 1.3, 0.27
    lam = 2 * mu * nu / (1 - 2 * nu)

    def traction(field, x, y, nx, ny, s, h=1e-5):
        G = np.zeros((3, 3))
        for j in range(3):
            e = np.zeros(3)
            e[j] = h
            up = oracle.kernel_tensor(field, x + e, y, np.zeros(3), ny, mu, nu) @ s
            um = oracle.kernel_tensor(field, x - e, y, np.zeros(3), ny, mu, nu) @ s
            G[:, j] = (up - um) / (2 * h)
        return (lam * np.trace(G) * np.eye(3) + mu * (G + G.T)) @ nx

    for kernel, field in (("ElasticHypersingular", "ElasticTraction"),
                          ("ElasticAdjointTraction", "ElasticDisplacement")):
        for _ in range(20):
            x = rng.normal(size=3)
            y = x + rng.normal(size=3) * 1.5
            nx, ny = rng.normal(size=3), rng.normal(size=3)
            nx /= np.linalg.norm(nx)
            ny /= np.linalg.norm(ny)
            s = rng.normal(size=3)
            direct = oracle.kernel_tensor(kernel, x, y, nx, ny, mu, nu) @ s
            assert np.linalg.norm(direct - traction(field, x, y, nx, ny, s)) <= 1e-7 * np.linalg.norm(direct)

