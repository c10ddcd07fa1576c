"""CPU tests of the nearfield construction's host side against the
reference's own outputs (tests/golden/nearfield_*.npz, made by the
reference's construction with oracle/ref/gte_restated.cpp standing in for the
absent GTEngine): the Galerkin observation points and their Richardson
(limit) directions bit for bit, the Gauss rules, and the argument checks.
No device compute happens here."""
import glob
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "nearfield_*.npz")))


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[10:-4] for p in CASES])
def test_obs_points_and_limit_directions_match_reference(path):
    from tbempy import ThreeD
    g = dict(np.load(path))
    m = ThreeD.Mesh(g["vertices"], g["facets"])
    loc, nrm, dirs = ThreeD.galerkin_obs_points(m, m, int(g["obs_near_order"]))
    dim = m.dim
    assert np.array_equal(loc, g["obs_loc"][:, :dim])
    assert np.array_equal(dirs, g["obs_dir"][:, :dim])
    # points on the surface step off it: every direction is non-zero
    assert np.all(np.abs(dirs).sum(axis=1) > 0)


def test_gauss_rules_integrate_polynomials():
    """gauss_facet: degree 2n - 1 on [-1, 1]; the collapsed tensor rule on
    the unit triangle integrates x^a y^b exactly (a + b <= 2n - 2) -- to the
    1e-12 the reference's Newton iteration leaves (its weights for n = 20 sum
    to 2 - 2e-13)."""
    from math import factorial
    from tbempy import ThreeD
    for n in (1, 3, 7, 20):
        x, w = ThreeD.gauss_facet(2, n)
        for k in range(2 * n):
            exact = 0.0 if k % 2 else 2.0 / (k + 1)
            assert abs((w * x[:, 0] ** k).sum() - exact) < 1e-12
        x, w = ThreeD.gauss_facet(3, n)
        assert len(w) == n * n
        for a in range(n):
            for b in range(n - 1 - a + 1):
                if a + b > 2 * n - 2:
                    continue
                exact = factorial(a) * factorial(b) / factorial(a + b + 2)
                assert abs((w * x[:, 0] ** a * x[:, 1] ** b).sum() - exact) < 1e-12


def test_gauss_rules_match_reference():
    from oracle import oracle
    from tbempy import ThreeD
    if not os.path.isdir(os.path.join(oracle.REF_ROOT, "cpp")):
        pytest.skip("reference checkout absent")
    if not oracle.ref_available():
        pytest.skip("reference library not built here")
    for dim in (2, 3):
        for n in (1, 2, 5, 12, 33):
            a, b = ThreeD.gauss_facet(dim, n), oracle.ref_gauss_facet(dim, n)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_bad_facet_indices_refused():
    from tbempy import ThreeD
    from tbempy._lib import TbemError
    g = dict(np.load(CASES[0]))
    m = ThreeD.Mesh(g["vertices"], g["facets"])
    with pytest.raises(TbemError):
        ThreeD.galerkin_obs_points(ThreeD.Mesh(m.vertices, m.facets + 10 * len(m.vertices)), m, 2)


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[10:-4] for p in CASES])
def test_galerkin_and_interpolation_operators_match_reference(path):
    """The host assembly of the Galerkin and interpolation operators against
    the reference's make_galerkin_operator / make_interpolation_operator
    (same layout; values to the last bit or one rounding)."""
    from oracle import oracle
    from tbempy import ThreeD
    if not oracle.ref_available():
        pytest.skip("reference library not built here")
    g = dict(np.load(path))
    m = ThreeD.Mesh(g["vertices"], g["facets"])
    for ncomp in (1, m.dim):
        for order in (2, 3):
            for which, fn in ((0, ThreeD.galerkin_csr), (1, ThreeD.interpolation_csr)):
                nr, nc, vals, cols, rows = fn(ncomp, m, order)
                rr, rc, rv, rcols, rrows = oracle.ref_galerkin_interp(which, g["vertices"], g["facets"],
                                                                      ncomp, order)
                assert (nr, nc) == (rr, rc)
                assert np.array_equal(rows, rrows) and np.array_equal(cols, rcols)
                assert np.allclose(vals, rv, rtol=2e-16, atol=0)


def test_nearfield_create_validates_before_device_use():
    """Bad kernel ids, integrator parameters, `which` and facet indices come
    back as TBEM_ERR_ARG with a message, before anything touches the device."""
    import ctypes as C
    from tbempy import _lib
    L = _lib.lib()
    v = np.ascontiguousarray([[0, 0, 0], [1, 0, 0], [0, 1, 0]], dtype=np.float64)
    f = np.ascontiguousarray([[0, 1, 2]], dtype=np.int64)
    bad_f = np.ascontiguousarray([[0, 1, 7]], dtype=np.int64)
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    good = _lib.TbemIntegrator(0, 0.0, 5, 2, 2, 2, 8, 3.0)
    cases = [
        (42, f, good, 0, "kernel"),                                        # unknown kernel
        (1, f, good, 5, "which"),                                          # bad which
        (1, f, _lib.TbemIntegrator(0, 0.0, 0, 2, 2, 2, 8, 3.0), 0, "integrator"),  # sinh order 0
        (1, f, _lib.TbemIntegrator(1, 0.0, 0, 2, 2, 2, 8, 3.0), 0, "integrator"),  # adaptive tol 0
        (1, f, _lib.TbemIntegrator(7, 1e-4, 5, 2, 2, 2, 8, 3.0), 0, "strategy"),
        (1, f, _lib.TbemIntegrator(0, 0.0, 5, 2, 2, 2, 1, 3.0), 0, "integrator"),  # < 2 steps
        (1, f, _lib.TbemIntegrator(0, 0.0, 5, 2, 2, 2, 8, -1.0), 0, "integrator"),
        (1, bad_f, good, 0, "index"),                                      # vertex out of range
    ]
    for kid, fac, cfg, which, word in cases:
        h = C.c_void_p()
        rc = L.tbem_nearfield_create(kid, None, P(v), 3, P(fac), 1, P(fac), 1, P(fac), 1,
                                     C.byref(cfg), which, C.byref(h))
        assert rc == -1, (kid, which)
        assert word in L.tbem_last_error().decode(), L.tbem_last_error()
        assert not h.value
    # null vertex / facet arrays with a nonzero count are argument errors, not crashes
    h = C.c_void_p()
    rc = L.tbem_nearfield_create(1, None, None, 3, P(f), 1, P(f), 1, P(f), 1, C.byref(good), 0,
                                 C.byref(h))
    assert rc == -1 and "null" in L.tbem_last_error().decode()
    rc = L.tbem_nearfield_create(1, None, P(v), 3, None, 1, P(f), 1, P(f), 1, C.byref(good), 0,
                                 C.byref(h))
    assert rc == -1 and "null" in L.tbem_last_error().decode() and not h.value
    # a point on a source facet with no limit direction (all_facets far away)
    # cannot take the sinh rule (the reference asserts): refused by the host
    # plan, before any device use
    allv = np.ascontiguousarray([[0, 0, 0], [1, 0, 0], [0, 1, 0], [50, 0, 0], [51, 0, 0], [50, 1, 0]],
                                dtype=np.float64)
    src_f = np.ascontiguousarray([[0, 1, 2]], dtype=np.int64)
    far_f = np.ascontiguousarray([[3, 4, 5]], dtype=np.int64)
    p = np.ascontiguousarray([[0.0, 0.0, 0.0]])  # a corner: distance exactly 0
    pn = np.ascontiguousarray([[0.0, 0.0, 1.0]])
    rc = L.tbem_nearfield_points_create(1, None, P(p), P(pn), 1, P(allv), 6, P(src_f), 1, P(far_f), 1,
                                        C.byref(good), 0, C.byref(h))
    assert rc == -1 and "lies on a source facet" in L.tbem_last_error().decode() and not h.value
    assert L.tbem_galerkin_obs_points(3, P(v), 3, None, 1, P(f), 1, 2, None, None, None) == -1
    assert L.tbem_interior_obs_points(3, P(v), 1, P(v), 3, None, 1, None) == -1
    assert L.tbem_gauss_facet(4, 3, None, None) == -1
    assert "dim" in L.tbem_last_error().decode()
    assert L.tbem_gauss_facet(3, 0, None, None) == -1


INTERIOR = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "interior_*.npz")))


@pytest.mark.parametrize("path", INTERIOR, ids=[os.path.basename(p)[9:-4] for p in INTERIOR])
def test_interior_limit_directions_and_mass_operator_match_reference(path):
    """dense_interior_operator's observation points (interior_obs_pts: points
    on the surface, just off it, inside and far) get the reference's limit
    directions bit for bit; mass_operator_scalar / _tensor equal the
    reference's (cpp/mass_operator.h) in layout and value."""
    from tbempy import ThreeD
    g = dict(np.load(path))
    m = ThreeD.Mesh(g["vertices"], g["facets"])
    assert np.array_equal(ThreeD.interior_limit_directions(g["locs"], m), g["dirs"])
    for R in sorted({1, m.dim}):
        for nq in (2, 3):
            nr, nc, vals, cols, rows = ThreeD.mass_csr(R, m, nq)
            key = "mass_%d_%d_" % (R, nq)
            assert (nr, nc) == tuple(g[key + "shape"])
            assert np.array_equal(rows, g[key + "rowptr"]) and np.array_equal(cols, g[key + "cols"])
            assert np.allclose(vals, g[key + "values"], rtol=1e-15, atol=0)


def test_dense_operator_host_side():
    """DenseOperator (cpp/dense_operator.h:11-40): shape, data(), to_dense,
    clone, size check; nothing reaches the device before an apply."""
    from tbempy import ThreeD
    d = np.arange(12.0)
    A = ThreeD.DenseOperator(3, 4, d)
    assert (A.n_rows(), A.n_cols(), A.n_elements()) == (3, 4, 12)
    assert np.array_equal(A.data(), d) and np.array_equal(A.to_dense(), d.reshape(3, 4))
    assert np.array_equal(A.clone().data(), d)
    with pytest.raises(ValueError):
        ThreeD.DenseOperator(3, 5, d)


@pytest.mark.parametrize("kernel,dim,n_terms", [(0, 3, 6), (1, 3, 6), (3, 3, 6), (6, 3, 6),
                                                (16, 2, 6), (19, 2, 6), (22, 2, 6),
                                                (1, 3, 160), (17, 2, 600)])
def test_adaptive_engine_matches_reference(kernel, dim, n_terms, tmp_path):
    """The level-by-level adaptive Gauss-Lobatto engine the product drives
    (3bem_gb300/csrc/nearfield_adaptive.cpp), run here with the oracle's CPU
    kernels as its point evaluator (tests/cpp/adaptive_driver.cpp; the product
    evaluates the same points on the GPU), equals the reference's recursive
    integrator (cpp/adaptive_quad.h via compute_term) bit for bit on near
    terms; the larger cases spread the terms over several host chunks."""
    import subprocess
    from oracle import oracle
    if not os.path.isdir(os.path.join(oracle.REF_ROOT, "cpp")):
        pytest.skip("reference checkout absent")
    if not oracle.ref_available():
        pytest.skip("reference library not built here")
    exe = str(tmp_path / "adaptive_driver")
    csrc = os.path.join(ROOT, "3bem_gb300", "csrc")
    odir = os.path.join(ROOT, "oracle")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + csrc,
                           "-I" + os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "adaptive_driver.cpp"),
                           os.path.join(csrc, "nearfield_adaptive.cpp"),
                           os.path.join(csrc, "nearfield_host.cpp"), "-o", exe,
                           os.path.join(odir, "liboracle.so"), "-Wl,-rpath," + odir])
    rng = np.random.default_rng(kernel)
    facet = (np.array([[0, 0, 0], [1.0, 0.1, 0], [0.2, 0.9, 0.1]]) if dim == 3
             else np.array([[0, 0, 0], [1.0, 0.2, 0]]))
    tol = 1e-5
    terms = []
    for _ in range(n_terms):
        obs = facet.mean(axis=0) + rng.normal(size=3) * 0.3
        n = rng.normal(size=3)
        if dim == 2:
            obs[2] = n[2] = 0.0
        terms.append((obs, n / np.linalg.norm(n)))
    lines = ["%d %.17g %.17g %.17g %d" % (kernel, 1.3, 0.27, tol, dim)]
    for obs, n in terms:
        lines.append(" ".join("%.17g" % v for v in list(obs) + list(n) + list(facet.ravel())))
    out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True,
                         check=True).stdout.strip().split("\n")
    for (obs, n), row in zip(terms, out):
        mine = np.array([float(v) for v in row.split()])
        ref = oracle.ref_term(kernel, obs[:dim], n[:dim], np.zeros(dim), facet[:, :dim], "adaptive",
                              tol, 0, 2, 2, 2, 8, 1e9, 1.3, 0.27).ravel()
        assert np.array_equal(mine, ref)
    if n_terms > 6:  # terms and inner integrals in small slices: the same values
        for slice_jobs in ("7", "50"):
            sliced = subprocess.run([exe, slice_jobs], input="\n".join(lines) + "\n", capture_output=True,
                                    text=True, check=True).stdout.strip().split("\n")
            assert sliced == out



@pytest.fixture(scope="module")
def plan_driver(tmp_path_factory):
    import subprocess
    from oracle import oracle
    oracle.build()
    exe = str(tmp_path_factory.mktemp("plan") / "nearfield_plan_driver")
    csrc = os.path.join(ROOT, "3bem_gb300", "csrc")
    odir = os.path.join(ROOT, "oracle")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + csrc,
                           os.path.join(ROOT, "tests", "cpp", "nearfield_plan_driver.cpp"),
                           os.path.join(csrc, "nearfield_host.cpp"), "-o", exe, "-lpthread",
                           os.path.join(odir, "liboracle.so"), "-Wl,-rpath," + odir])
    return exe


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[10:-4] for p in CASES])
def test_term_plan_and_csr_layout_match_reference(path, plan_driver):
    """The host plan of both matrices (the terms in the reference's order,
    their far / near / singular split and evaluations, the Richardson and
    negation step and the CSR layout: nearfield_host.cpp plan_terms and
    assemble_csr) reproduces the reference's row pointers and columns; with
    the far evaluations done on the CPU by the oracle's kernels in the
    reference's summation order, the correction matrix's values equal the
    reference's bit for bit (the product evaluates the same items on the
    GPU, lanes summing in a different order)."""
    import subprocess
    from oracle import oracle
    g = dict(np.load(path))
    dim = g["facets"].shape[1]
    verts = np.zeros((len(g["vertices"]), 3))
    verts[:, :g["vertices"].shape[1]] = g["vertices"]
    for which in (0, 1):
        order = int(g["obs_near_order"] if which == 0 else g["obs_far_order"])
        head = "%d %.17g %.17g %d %d %.17g %d %d %d" % (
            oracle.kernel_id(str(g["kernel"]), dim), float(g["mu"]), float(g["nu"]), dim, order,
            float(g["far_threshold"]),
            int(g["n_singular_steps"]), int(g["src_far_order"]), which)
        lines = [head, str(len(verts))] + ["%.17g %.17g %.17g" % tuple(v) for v in verts]
        lines += [str(len(g["facets"]))] + [" ".join(str(int(i)) for i in f) for f in g["facets"]]
        out = subprocess.run([plan_driver], input="\n".join(lines) + "\n", capture_output=True,
                             text=True, check=True).stdout.split("\n")
        n_rows, n_cols, nnz = (int(x) for x in out[0].split())
        assert (n_rows, n_cols) == tuple(g["shape%d" % which])
        assert np.array_equal(np.array(out[1].split(), dtype=np.int64), g["rowptr%d" % which])
        assert np.array_equal(np.array(out[2].split(), dtype=np.int64), g["cols%d" % which])
        if which == 1:
            assert np.array_equal(np.array(out[3].split(), dtype=np.float64), g["values1"])
