"""GPU parity of the nearfield and farfield-correction matrices with the
reference's own construction (tests/golden/nearfield_*.npz: 3D and 2D
meshes, Laplace and elastic kernels including the hypersingular ones,
Richardson extrapolation for the on-surface observation points; the sinh
strategy and the adaptive Gauss-Lobatto one).

Tolerance (written here, checked below): max |GPU - reference| <= max(1e-10,
100 x floor) x max |reference entry|, with floor the reference's own change
when every vertex moves by one ulp (stored in the fixture: <= 1e-13 for the
3D cases, 1.4e-10 for the 2D cases whose Richardson extrapolation cancels
the most).  Same layout: identical row pointers and column indices (the
reference's facet order is reproduced).
"""
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "nearfield_*.npz")))


def dense(shape, vals, cols, rows):
    a = np.zeros(tuple(shape))
    for r in range(shape[0]):
        np.add.at(a[r], cols[rows[r]:rows[r + 1]], vals[rows[r]:rows[r + 1]])
    return a


def kernel_of(g, dim):
    from tbempy import ThreeD, TwoD
    k = getattr(TwoD if dim == 2 else ThreeD, str(g["kernel"]))
    return k(float(g["mu"]), float(g["nu"])) if str(g["kernel"]).startswith("Elastic") else k()


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[10:-4] for p in CASES])
def test_nearfield_matrices_match_reference(path):
    from tbempy import ThreeD
    g = dict(np.load(path))
    m = ThreeD.Mesh(g["vertices"], g["facets"])
    rest = (int(g["obs_near_order"]), int(g["obs_far_order"]), int(g["src_far_order"]),
            int(g["n_singular_steps"]), float(g["far_threshold"]), kernel_of(g, m.dim))
    if str(g["strategy"]) == "adaptive":
        mthd = ThreeD.make_adaptive_integrator(float(g["near_tol"]), *rest)
    else:
        mthd = ThreeD.make_sinh_integrator(int(g["sinh_order"]), *rest)
    for which, build in ((0, ThreeD.nearfield_operator), (1, ThreeD.farfield_correction_operator)):
        op = build(m, m, mthd, m)
        assert (op.n_rows(), op.n_cols()) == tuple(g["shape%d" % which])
        assert np.array_equal(op.row_ptrs(), g["rowptr%d" % which])
        assert np.array_equal(op.column_indices(), g["cols%d" % which])
        ref = g["values%d" % which]
        tol = max(1e-10, 100 * float(g["ulp_floor%d" % which])) * np.abs(ref).max()
        assert np.abs(op.values() - ref).max() <= tol
        # the device CSR applies the same matrix
        x = np.random.default_rng(1).uniform(-1, 1, op.n_cols())
        A = dense(g["shape%d" % which], ref, g["cols%d" % which], g["rowptr%d" % which])
        assert np.linalg.norm(op.apply(x) - A @ x) <= 1e-8 * np.linalg.norm(A @ x) + 1e-300


def test_boundary_operator_assembles_and_matches_dense_chain():
    """boundary_operator: the device chain G_near N + G_far C + G_far F I with
    the FMM farfield equals the same chain with the direct farfield."""
    from tbempy import ThreeD, meshes
    v, f = meshes.icosphere(2)
    m = ThreeD.Mesh(v, f)
    K = ThreeD.LaplaceDouble()
    mthd = ThreeD.make_sinh_integrator(5, 3, 3, 3, 8, 3.0, K)
    A = ThreeD.boundary_operator(m, m, mthd, ThreeD.FMMConfig(0.3, 75, 20, 0.05, False), m)
    assert A.n_rows() == m.n_dofs() and A.n_cols() == m.n_dofs()
    x = np.random.default_rng(2).uniform(-1, 1, m.n_dofs())
    y = A.apply(x)
    ol, on, _ = ThreeD.quadrature_points(m, 3)
    sl, sn, sw = ThreeD.quadrature_points(m, 3)
    D = ThreeD.DirectOperator(K, ol, on, sl, sn, sw)
    chain = ThreeD.IntegralOperator(A.nearfield, A.farfield_correction, A.galerkin, D, A.interp)
    yd = chain.apply(x)
    assert np.linalg.norm(y - yd) <= 1e-6 * np.linalg.norm(yd)
    # the double layer of a constant density on a closed surface, its limit
    # taken along the facet normals (outward here): the exterior value 0 (the
    # reference's own matrices give |A 1| <= 2.4e-3 of the basis integrals)
    ones = np.ones(m.n_dofs())
    g = A.galerkin.apply(np.ones(A.galerkin.n_cols()))  # integrals of the basis functions
    assert np.abs(A.apply(ones)).max() <= 5e-3 * np.abs(g).max()


INTERIOR = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "interior_*.npz")))


@pytest.mark.parametrize("path", INTERIOR, ids=[os.path.basename(p)[9:-4] for p in INTERIOR])
def test_interior_operator_matches_reference(path):
    """dense_interior_operator: its nearfield and correction matrices against
    the reference's (same tolerance as above); its apply against the
    reference's own dense operator applied to the same density
    (cpp/integral_operator.h:133-158), within max(1e-10, 100 x the one-ulp
    sensitivity of that apply); and against N x + C x + F (I x) with F the
    FP64 direct sum of the oracle (to 1e-10 of the contributions' size)."""
    from oracle import oracle
    from tbempy import ThreeD
    g = dict(np.load(path))
    m = ThreeD.Mesh(g["vertices"], g["facets"])
    K = kernel_of(g, m.dim)
    mthd = ThreeD.make_sinh_integrator(int(g["sinh_order"]), int(g["obs_near_order"]),
                                       int(g["obs_far_order"]), int(g["src_far_order"]),
                                       int(g["n_singular_steps"]), float(g["far_threshold"]), K)
    A = ThreeD.dense_interior_operator(g["locs"], g["normals"], m, mthd, m)
    for which, op in ((0, A.nearfield), (1, A.farfield_correction)):
        assert (op.n_rows(), op.n_cols()) == tuple(g["shape%d" % which])
        assert np.array_equal(op.row_ptrs(), g["rowptr%d" % which])
        assert np.array_equal(op.column_indices(), g["cols%d" % which])
        ref = g["values%d" % which]
        tol = max(1e-10, 100 * float(g["ulp_floor%d" % which])) * np.abs(ref).max()
        assert np.abs(op.values() - ref).max() <= tol
    x = g["apply_x"]
    y_ref = g["apply_y"]
    bar = max(1e-10, 100 * float(g["apply_ulp_floor"]))
    assert np.linalg.norm(A.apply(x) - y_ref) <= bar * np.linalg.norm(y_ref)
    N = dense(g["shape0"], g["values0"], g["cols0"], g["rowptr0"])
    Cc = dense(g["shape1"], g["values1"], g["cols1"], g["rowptr1"])
    I = A.interp
    Id = dense((I.n_rows(), I.n_cols()), I.values(), I.column_indices(), I.row_ptrs())
    sl, sn, sw = ThreeD.quadrature_points(m, int(g["src_far_order"]))
    far = oracle.direct(K.kernel_id, g["locs"], g["normals"], sl, sn, sw, Id @ x,
                        mu=float(g["mu"]), nu=float(g["nu"]))
    expect = N @ x + Cc @ x + far
    # points 1e-4 off the surface sit next to source quadrature points: their
    # farfield and its correction are ~3e5 and cancel to O(1) (a different
    # summation order alone moves the total by 3e-10 of it), so the bound is
    # relative to the size of the contributions; measured on GB300: 1.3e-12
    scale = np.linalg.norm(N @ x) + np.linalg.norm(Cc @ x) + np.linalg.norm(far)
    assert np.linalg.norm(A.apply(x) - expect) <= 1e-10 * scale


DENSE = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "dense_boundary_*.npz")))


@pytest.mark.parametrize("path", DENSE, ids=[os.path.basename(p)[15:-4] for p in DENSE])
def test_dense_boundary_operator_matches_reference(path):
    """dense_boundary_operator against the reference's own dense assembly
    (cpp/integral_operator.h:100-130; its composition with the reference's
    parts reproduces the fixture to 3e-16 on the CPU): within max(1e-9, 100 x
    the reference's one-ulp sensitivity) of the largest entry, and its GPU
    apply equals the dense product."""
    from tbempy import ThreeD
    g = dict(np.load(path))
    m = ThreeD.Mesh(g["vertices"], g["facets"])
    mthd = ThreeD.make_sinh_integrator(int(g["sinh_order"]), int(g["obs_near_order"]),
                                       int(g["obs_far_order"]), int(g["src_far_order"]),
                                       int(g["n_singular_steps"]), float(g["far_threshold"]),
                                       kernel_of(g, m.dim))
    A = ThreeD.dense_boundary_operator(m, m, mthd, m)
    ref = g["matrix"]
    M = A.to_dense()
    assert M.shape == ref.shape
    assert np.abs(M - ref).max() <= max(1e-9, 100 * float(g["ulp_floor"])) * np.abs(ref).max()
    x = np.random.default_rng(4).uniform(-1, 1, A.n_cols())
    assert np.linalg.norm(A.apply(x) - M @ x) <= 1e-12 * np.linalg.norm(M @ x)
