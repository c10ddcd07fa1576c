"""Boundary-operator assembly around the apply, with the reference's names.

The reference builds a Galerkin boundary operator as
``boundary_operator(obs_mesh, src_mesh, mthd, fmm_config, all_mesh)``
(cpp/integral_operator.h:66-99):

    A = G_near N + G_far C + G_far F I

with N the nearfield matrix and C the farfield correction
(cpp/nearfield_operator.h:97-117), G the Galerkin operators
(cpp/galerkin_operator.cpp:9-44), I the interpolation operator
(cpp/interpolation_operator.cpp:9-39) and F the farfield N-body operator
over the quadrature points (``nbody_data_from_bem``,
cpp/nbody_operator.h:40-85).  Here N and C are integrated on the GPU
(``tbem_nearfield_create``), F is the GPU FMM (the reference left its FMM
farfield commented out and applied a dense operator), and the whole chain
is applied on the device by ``IntegralOperator``.

Meshes are ``Mesh(vertices [n, dim], facets [m, dim])``; the strategy comes
from ``make_sinh_integrator`` or ``make_adaptive_integrator``
(cpp/integral_term.h:53-150): sinh-transformed Gauss rules, or the adaptive
Gauss-Lobatto rule (cpp/adaptive_quad.h) whose subdivision the host decides
level by level while the GPU evaluates every level's points.
"""
import ctypes as C

import numpy as np

from . import _lib as _L
from ._lib import check
from .ThreeD import FMMConfig, FMMOperator, IntegralOperator, SparseOperator, _ptr  # noqa: F401


class Mesh:
    """Facets over shared vertices (Mesh<dim>::from_vertices_faces,
    cpp/mesh.cpp:175-188): vertices [n, dim], facets [m, dim] indices."""

    def __init__(self, vertices, facets):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float64)
        self.dim = self.vertices.shape[1]
        self.facets = np.ascontiguousarray(np.asarray(facets, dtype=np.int64).reshape(-1, self.dim))

    def n_facets(self):
        return len(self.facets)

    def n_dofs(self):
        return self.dim * len(self.facets)

    def corners(self):
        """[m, dim, dim]: the facets' corner coordinates."""
        return self.vertices[self.facets]


class IntegrationStrategy:
    """The arguments of make_sinh_integrator / make_adaptive_integrator
    (cpp/integral_term.h:53-150) with the kernel."""

    def __init__(self, kind, K, near_tol, sinh_order, obs_near_order, obs_far_order,
                 src_far_order, n_singular_steps, far_threshold):
        self.kind = kind
        self.K = K
        self.near_tol = near_tol
        self.sinh_order = int(sinh_order)
        self.obs_near_order = int(obs_near_order)
        self.obs_far_order = int(obs_far_order)
        self.src_far_order = int(src_far_order)
        self.n_singular_steps = int(n_singular_steps)
        self.far_threshold = float(far_threshold)

    def _c(self):
        return _L.TbemIntegrator(1 if self.kind == "adaptive" else 0, float(self.near_tol or 0.0),
                                 self.sinh_order, self.obs_near_order, self.obs_far_order,
                                 self.src_far_order, self.n_singular_steps, self.far_threshold)


def make_sinh_integrator(sinh_order, obs_near_order, obs_far_order, src_far_order,
                         n_singular_steps, far_threshold, K):
    return IntegrationStrategy("sinh", K, 0.0, sinh_order, obs_near_order, obs_far_order,
                               src_far_order, n_singular_steps, far_threshold)


def make_adaptive_integrator(near_tol, obs_near_order, obs_far_order, src_far_order,
                             n_singular_steps, far_threshold, K):
    return IntegrationStrategy("adaptive", K, near_tol, 0, obs_near_order, obs_far_order,
                               src_far_order, n_singular_steps, far_threshold)


def gauss_facet(dim, n):
    """(x [n, dim - 1], w [n]): the reference facet's Gauss rule."""
    L = _L.lib()
    k = check(L.tbem_gauss_facet(int(dim), int(n), None, None))
    x = np.zeros((k, dim - 1))
    w = np.zeros(k)
    check(L.tbem_gauss_facet(int(dim), int(n), _ptr(x), _ptr(w)))
    return x, w


def _merge(*meshes):
    """One vertex array for several meshes and their facets re-indexed into it."""
    verts = np.ascontiguousarray(np.concatenate([m.vertices for m in meshes]))
    out, off = [], 0
    for m in meshes:
        out.append(np.ascontiguousarray(m.facets + off))
        off += len(m.vertices)
    return verts, out


def galerkin_obs_points(obs_mesh, all_mesh, order):
    """Observation points, normals and Richardson directions (each [n, dim])."""
    dim = obs_mesh.dim
    v, (of, af) = _merge(obs_mesh, all_mesh)
    L = _L.lib()
    n = check(L.tbem_galerkin_obs_points(dim, _ptr(v), len(v), _ptr(of), len(of), _ptr(af), len(af),
                                         int(order), None, None, None))
    locs, nrm, dirs = (np.zeros((n, dim)) for _ in range(3))
    check(L.tbem_galerkin_obs_points(dim, _ptr(v), len(v), _ptr(of), len(of), _ptr(af), len(af),
                                     int(order), _ptr(locs), _ptr(nrm), _ptr(dirs)))
    return locs, nrm, dirs


def _nearfield(obs_mesh, src_mesh, mthd, all_mesh, which):
    if mthd.K.space_dim != obs_mesh.dim:
        raise ValueError("the kernel's dimension does not match the mesh's")
    v, (of, sf, af) = _merge(obs_mesh, src_mesh, all_mesh)
    h = C.c_void_p()
    cfg = mthd._c()
    check(_L.lib().tbem_nearfield_create(mthd.K.kernel_id, _ptr(mthd.K.params()), _ptr(v), len(v),
                                         _ptr(of), len(of), _ptr(sf), len(sf), _ptr(af), len(af),
                                         C.byref(cfg), int(which), C.byref(h)))
    return SparseOperator._from_handle(h)


def nearfield_operator(obs_mesh, src_mesh, mthd, all_mesh):
    """make_nearfield_operator(galerkin_obs_pts(obs_mesh, obs_near_quad,
    all_mesh), src_mesh, mthd) (cpp/nearfield_operator.h:97-106)."""
    return _nearfield(obs_mesh, src_mesh, mthd, all_mesh, 0)


def farfield_correction_operator(obs_mesh, src_mesh, mthd, all_mesh):
    """make_farfield_correction_operator with the far observation points
    (cpp/nearfield_operator.h:108-117)."""
    return _nearfield(obs_mesh, src_mesh, mthd, all_mesh, 1)


def _jacobians(mesh):
    c = mesh.corners()
    if mesh.dim == 2:
        d = c[:, 1] - c[:, 0]
        return 0.5 * np.sqrt(d[:, 0] ** 2 + d[:, 1] ** 2)
    n = np.cross(c[:, 2] - c[:, 0], c[:, 2] - c[:, 1])
    return 2.0 * (0.5 * np.sqrt((n * n).sum(axis=1)))


def _basis(x, dim):
    if dim == 2:
        return np.stack([0.5 - 0.5 * x[:, 0], 0.5 + 0.5 * x[:, 0]], axis=1)
    return np.stack([1 - x[:, 0] - x[:, 1], x[:, 0], x[:, 1]], axis=1)


def _csr_arrays(n_rows, n_cols, rows, cols, vals):
    """csr_from_coo (cpp/sparse_operator.cpp:140-172): entries keep their input
    order inside a row.  Returns (n_rows, n_cols, values, column_indices, row_ptrs)."""
    order = np.argsort(rows, kind="stable")
    counts = np.bincount(rows, minlength=n_rows)
    return (n_rows, n_cols, vals[order], cols[order].astype(np.int64),
            np.concatenate([[0], np.cumsum(counts)]).astype(np.int64))


def galerkin_csr(n_components, obs_mesh, order):
    """make_galerkin_operator (cpp/galerkin_operator.cpp:9-44) as host CSR
    arrays: rows d * n_dofs + dof, columns d * n_quad_points + quad point,
    values basis * (jacobian * weight)."""
    dim = obs_mesh.dim
    x, w = gauss_facet(dim, order)
    nq, nf = len(w), obs_mesh.n_facets()
    bas = _basis(x, dim)
    jac = _jacobians(obs_mesh)
    f, q, b, d = np.meshgrid(np.arange(nf), np.arange(nq), np.arange(dim), np.arange(n_components),
                             indexing="ij")
    rows = d * obs_mesh.n_dofs() + dim * f + b
    cols = d * (nf * nq) + f * nq + q
    vals = bas[q, b] * (jac[f] * w[q])
    return _csr_arrays(n_components * obs_mesh.n_dofs(), n_components * nf * nq, rows.ravel(),
                       cols.ravel(), vals.ravel())


def galerkin_operator(n_components, obs_mesh, order):
    """make_galerkin_operator as a GPU SparseOperator."""
    return SparseOperator(*galerkin_csr(n_components, obs_mesh, order))


def interpolation_csr(n_components, src_mesh, order):
    """make_interpolation_operator (cpp/interpolation_operator.cpp:9-39) as
    host CSR arrays."""
    dim = src_mesh.dim
    x, w = gauss_facet(dim, order)
    nq, nf = len(w), src_mesh.n_facets()
    bas = _basis(x, dim)
    f, q, b, d = np.meshgrid(np.arange(nf), np.arange(nq), np.arange(dim), np.arange(n_components),
                             indexing="ij")
    rows = d * (nf * nq) + f * nq + q
    cols = d * src_mesh.n_dofs() + dim * f + b
    vals = bas[q, b]
    return _csr_arrays(n_components * nf * nq, n_components * src_mesh.n_dofs(), rows.ravel(),
                       cols.ravel(), vals.ravel())


def interpolation_operator(n_components, src_mesh, order):
    """make_interpolation_operator as a GPU SparseOperator."""
    return SparseOperator(*interpolation_csr(n_components, src_mesh, order))


def quadrature_points(mesh, order):
    """(locs, normals, weights) of the facets' Gauss points
    (nbody_obs_from_bem / nbody_src_from_bem, cpp/nbody_operator.h:36-72)."""
    dim = mesh.dim
    x, w = gauss_facet(dim, order)
    c = mesh.corners()
    bas = _basis(x, dim)
    # ref_to_real (cpp/numerics.h:81-100): the basis dotted with the corners
    # left to right, each product rounded -- the positions the nearfield
    # construction's far rule uses too (nearfield.cu: influence), so a
    # farfield and its correction cancel to rounding of their own size
    locs = bas[None, :, 0, None] * c[:, None, 0, :]
    for b in range(1, dim):
        locs = locs + bas[None, :, b, None] * c[:, None, b, :]
    locs = locs.reshape(-1, dim)
    if dim == 2:
        d = c[:, 1] - c[:, 0]
        n = np.stack([-d[:, 1], d[:, 0]], axis=1)
    else:
        n = np.cross(c[:, 2] - c[:, 0], c[:, 2] - c[:, 1])
    n = n * (1 / np.sqrt((n * n).sum(axis=1)))[:, None]
    normals = np.repeat(n, len(w), axis=0)
    weights = (w[None, :] * _jacobians(mesh)[:, None]).ravel()
    return np.ascontiguousarray(locs), np.ascontiguousarray(normals), weights


def _product(A, B):
    """A B for two SparseOperators (SparseOperator::right_multiply,
    cpp/sparse_operator.cpp:114-138), assembled once at setup on the host."""
    import scipy.sparse as sp
    a = sp.csr_matrix((A.values(), A.column_indices(), A.row_ptrs()), shape=(A.n_rows(), A.n_cols()))
    b = sp.csr_matrix((B.values(), B.column_indices(), B.row_ptrs()), shape=(B.n_rows(), B.n_cols()))
    p = (a @ b).tocsr()
    p.sort_indices()
    return SparseOperator(p.shape[0], p.shape[1], p.data, p.indices.astype(np.int64),
                          p.indptr.astype(np.int64))


def boundary_operator(obs_mesh, src_mesh, mthd, fmm_config, all_mesh, precision="fp64"):
    """The Galerkin boundary operator A = G_near N + G_far C + G_far F I
    (cpp/integral_operator.h:66-99) with the GPU FMM as F."""
    K = mthd.K
    R = K.tensor_dim
    near = nearfield_operator(obs_mesh, src_mesh, mthd, all_mesh)
    corr = farfield_correction_operator(obs_mesh, src_mesh, mthd, all_mesh)
    g_near = galerkin_operator(R, obs_mesh, mthd.obs_near_order)
    g_far = galerkin_operator(R, obs_mesh, mthd.obs_far_order)
    interp = interpolation_operator(R, src_mesh, mthd.src_far_order)
    ol, on, _ = quadrature_points(obs_mesh, mthd.obs_far_order)
    sl, sn, sw = quadrature_points(src_mesh, mthd.src_far_order)
    far = FMMOperator(K, ol, on, sl, sn, sw, fmm_config, precision=precision)
    return IntegralOperator(_product(g_near, near), _product(g_far, corr), g_far, far, interp)


def interior_limit_directions(locs, all_mesh):
    """Limit (Richardson) directions of given points against a mesh, as
    interior_obs_pts computes them (cpp/nearfield_operator.h:27-40); [n, dim]."""
    dim = all_mesh.dim
    locs = np.ascontiguousarray(locs, dtype=np.float64).reshape(-1, dim)
    af = np.ascontiguousarray(all_mesh.facets)
    dirs = np.zeros_like(locs)
    check(_L.lib().tbem_interior_obs_points(dim, _ptr(locs), len(locs), _ptr(all_mesh.vertices),
                                            len(all_mesh.vertices), _ptr(af), len(af), _ptr(dirs)))
    return dirs


def _nearfield_points(locs, normals, src_mesh, mthd, all_mesh, which):
    dim = src_mesh.dim
    locs = np.ascontiguousarray(locs, dtype=np.float64).reshape(-1, dim)
    normals = np.ascontiguousarray(normals, dtype=np.float64).reshape(-1, dim)
    v, (sf, af) = _merge(src_mesh, all_mesh)
    h = C.c_void_p()
    cfg = mthd._c()
    check(_L.lib().tbem_nearfield_points_create(
        mthd.K.kernel_id, _ptr(mthd.K.params()), _ptr(locs), _ptr(normals), len(locs), _ptr(v),
        len(v), _ptr(sf), len(sf), _ptr(af), len(af), C.byref(cfg), int(which), C.byref(h)))
    return SparseOperator._from_handle(h)


def _identity(n):
    return SparseOperator(n, n, np.ones(n), np.arange(n, dtype=np.int64),
                          np.arange(n + 1, dtype=np.int64))


def dense_interior_operator(locs, normals, src_mesh, mthd, all_mesh, fmm_config=None):
    """The field of a boundary density at given points
    (dense_interior_operator, cpp/integral_operator.h:132-158):
    A = N + C + F I, with N and C integrated on the GPU for the points (their
    limit directions taken against all_mesh) and F the direct N-body operator
    over the source quadrature points -- or the GPU FMM when fmm_config is
    given.  Applied matrix-free on the device (the name is the reference's;
    the reference returns the assembled dense matrix)."""
    K = mthd.K
    locs = np.ascontiguousarray(locs, dtype=np.float64).reshape(-1, src_mesh.dim)
    normals = np.ascontiguousarray(normals, dtype=np.float64).reshape(-1, src_mesh.dim)
    near = _nearfield_points(locs, normals, src_mesh, mthd, all_mesh, 0)
    corr = _nearfield_points(locs, normals, src_mesh, mthd, all_mesh, 1)
    interp = interpolation_operator(K.tensor_dim, src_mesh, mthd.src_far_order)
    sl, sn, sw = quadrature_points(src_mesh, mthd.src_far_order)
    if fmm_config is None:
        from .ThreeD import DirectOperator
        far = DirectOperator(K, locs, normals, sl, sn, sw)
    else:
        far = FMMOperator(K, locs, normals, sl, sn, sw, fmm_config)
    return IntegralOperator(near, corr, _identity(K.tensor_dim * len(locs)), far, interp)


def mass_csr(n_components, mesh, n_q):
    """mass_operator (cpp/mass_operator.h:10-19): the Galerkin operator times
    the interpolation operator on the same Gauss rule, as host CSR arrays."""
    import scipy.sparse as sp
    g = galerkin_csr(n_components, mesh, n_q)
    i = interpolation_csr(n_components, mesh, n_q)
    a = sp.csr_matrix((g[2], g[3], g[4]), shape=(g[0], g[1]))
    b = sp.csr_matrix((i[2], i[3], i[4]), shape=(i[0], i[1]))
    p = (a @ b).tocsr()
    p.sort_indices()
    return (p.shape[0], p.shape[1], p.data, p.indices.astype(np.int64), p.indptr.astype(np.int64))


def mass_operator_scalar(mesh, n_q):
    """mass_operator<dim,1,1> (python_wrapper/dimension.cpp:93)."""
    return SparseOperator(*mass_csr(1, mesh, n_q))


def mass_operator_tensor(mesh, n_q):
    """mass_operator<dim,dim,dim> (python_wrapper/dimension.cpp:94)."""
    return SparseOperator(*mass_csr(mesh.dim, mesh, n_q))


def _dense(csr):
    nr, nc, vals, cols, rows = csr
    out = np.zeros((nr, nc))
    for r in range(nr):
        np.add.at(out[r], cols[rows[r]:rows[r + 1]], vals[rows[r]:rows[r + 1]])
    return out


def dense_boundary_operator(obs_mesh, src_mesh, mthd, all_mesh):
    """The boundary operator assembled densely with the exact farfield
    (dense_boundary_operator, cpp/integral_operator.h:100-130):
    G_far (C + F I) + G_near N, F the direct N-body matrix over the
    quadrature points.  N and C are integrated on the GPU, F I is the GPU
    direct sum applied to the columns of I; the products are formed on the
    host.  Returns a DenseOperator (for small meshes, as in the reference)."""
    from .ThreeD import DenseOperator, DirectOperator
    K = mthd.K
    R = K.tensor_dim
    near = nearfield_operator(obs_mesh, src_mesh, mthd, all_mesh)
    corr = farfield_correction_operator(obs_mesh, src_mesh, mthd, all_mesh)
    g_near = _dense(galerkin_csr(R, obs_mesh, mthd.obs_near_order))
    g_far = _dense(galerkin_csr(R, obs_mesh, mthd.obs_far_order))
    interp = _dense(interpolation_csr(R, src_mesh, mthd.src_far_order))
    ol, on, _ = quadrature_points(obs_mesh, mthd.obs_far_order)
    sl, sn, sw = quadrature_points(src_mesh, mthd.src_far_order)
    F = DirectOperator(K, ol, on, sl, sn, sw)
    FI = np.asarray(F.apply(np.ascontiguousarray(interp.T))).T  # F applied to every column of I
    near_d = _dense((near.n_rows(), near.n_cols(), near.values(), near.column_indices(), near.row_ptrs()))
    corr_d = _dense((corr.n_rows(), corr.n_cols(), corr.values(), corr.column_indices(), corr.row_ptrs()))
    out = g_far @ (corr_d + FI) + g_near @ near_d
    return DenseOperator(out.shape[0], out.shape[1], out.ravel())

