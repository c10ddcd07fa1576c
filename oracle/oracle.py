"""ORACLE -- test infrastructure, not product code.

Python side of the CPU restatement of the reference KIFMM (fmm_oracle.cpp):
builds the shared library, computes the check-to-equivalent pseudo-inverses
with LAPACK dgesvd exactly as the reference's ``svd_pseudoinverse`` does
(cpp/blas_wrapper.cpp:67-127: the row-major matrix is handed to column-major
LAPACK, singular values <= 1e-10 * s_max are dropped, cpp/fmm.cpp:122), and
exposes the apply, the direct sum and the tree/list dumps.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline / reference
arm import this module, and only to check results.  ``RefLib`` wraps the
reference itself compiled from its own sources (oracle/_ref, built by
oracle/ref/Makefile where the reference checkout exists) to pin this
restatement.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import scipy.linalg

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libtbem_ref.so")

KERNELS = {"LaplaceSingle": 0, "LaplaceDouble": 1, "ElasticDisplacement": 2,
           "ElasticTraction": 3, "ElasticAdjointTraction": 4, "IdentityScalar": 5,
           "ElasticHypersingular": 6}
# 2D kernels (FMMOperator<2,1,1> / <2,2,2>); their points are [n][2] or [n][3]
# with z ignored
KERNELS_2D = {"LaplaceSingle": 16, "LaplaceDouble": 17, "LaplaceHypersingular": 18,
              "ElasticDisplacement": 19, "ElasticTraction": 20, "ElasticAdjointTraction": 21,
              "ElasticHypersingular": 22, "IdentityScalar": 23}
TENSOR_KERNELS = (2, 3, 4, 6)
TENSOR_KERNELS_2D = (19, 20, 21, 22)


def kernel_id(kernel, dim=3):
    if isinstance(kernel, str):
        return (KERNELS_2D if dim == 2 else KERNELS)[kernel]
    return int(kernel)


def kernel_components(k):
    """R (= C) of kernel id k."""
    return 3 if k in TENSOR_KERNELS else 2 if k in TENSOR_KERNELS_2D else 1


def space_dim(k):
    return 2 if k >= 16 else 3
LISTS = ["p2m", "m2m", "p2p", "m2p", "p2l", "m2l", "l2l", "l2p"]


def build(force=False):
    """Compile fmm_oracle.cpp (g++ -O3 -fopenmp, no FMA contraction)."""
    src = os.path.join(HERE, "fmm_oracle.cpp")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared",
                           "-ffp-contract=off", src, "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def _ref_root():
    """The reference checkout: $TBEM_REFERENCE_ROOT, else a folder named
    `reference` beside this repository, where one exists ("" when neither)."""
    env = os.environ.get("TBEM_REFERENCE_ROOT")
    if env:
        return env
    sib = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    return sib if os.path.isdir(os.path.join(sib, "cpp")) else ""


REF_ROOT = _ref_root()


def build_ref(ref_root=REF_ROOT):
    """Compile the reference's own sources into oracle/_ref (needs the checkout)."""
    if not os.path.isdir(os.path.join(ref_root, "cpp")):
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"),
                           "REF=" + ref_root, "-j8"])
    return REF_LIB_PATH


_P = C.c_void_p
_D = C.c_double
_L = C.c_long
_I = C.c_int


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _pts3(a):
    """[n][2] or [n][3] points as [n][3] (z = 0 added to 2D points)."""
    a = np.asarray(a, dtype=np.float64).reshape(len(a), -1)
    if a.shape[1] == 2:
        a = np.concatenate([a, np.zeros((len(a), 1))], axis=1)
    return np.ascontiguousarray(a)


def pinv_reference(A, threshold=1e-10):
    """Thresholded pseudo-inverse of a row-major square A, the reference way.

    LAPACK sees the row-major buffer as A^T (column-major); dgesvd gives
    A^T = U S V^T and the result is pinv(A) = U S^-1 V^T restricted to the
    singular values above threshold * s_max (cpp/blas_wrapper.cpp:109-169).
    """
    u, s, vt = scipy.linalg.svd(A.T, full_matrices=True, lapack_driver="gesvd")
    keep = s > threshold * s[0]
    return np.ascontiguousarray((u[:, keep] / s[keep]) @ vt[keep, :])


class _Lib:
    _cache = {}

    def __init__(self, path, prefix):
        self.lib = C.CDLL(path)
        self.prefix = prefix

    def fn(self, name, restype, argtypes):
        f = getattr(self.lib, self.prefix + name)
        f.restype = restype
        f.argtypes = argtypes
        return f


def _lib():
    if "oracle" not in _Lib._cache:
        _Lib._cache["oracle"] = _Lib(build(), "oracle_")
    return _Lib._cache["oracle"]


class _FMMBase:
    """Shared ctypes surface of the oracle and the reference shim."""

    def _setup(self, L, kernel, obs_locs, obs_normals, src_locs, src_normals,
               src_weights, mac, order, min_pts, d, small_cells, mu, nu):
        self.L = L
        dim = np.asarray(obs_locs).reshape(len(obs_locs), -1).shape[1] if len(obs_locs) else 3
        self.kernel = kernel_id(kernel, dim)
        self.R = kernel_components(self.kernel)
        self.obs_locs, self.obs_normals = _pts3(obs_locs), _pts3(obs_normals)
        self.src_locs, self.src_normals = _pts3(src_locs), _pts3(src_normals)
        self.src_weights = _f64(src_weights)
        self.n_obs, self.n_src = len(self.obs_locs), len(self.src_locs)
        create = L.fn("fmm_create" if L.prefix == "ref_" else "create", _P,
                      [_I, _D, _D, _P, _P, _L, _P, _P, _P, _L, _D, _L, _L, _D, _I])
        self.h = create(self.kernel, mu, nu, _ptr(self.obs_locs), _ptr(self.obs_normals),
                        self.n_obs, _ptr(self.src_locs), _ptr(self.src_normals),
                        _ptr(self.src_weights), self.n_src, mac, order, min_pts, d,
                        int(bool(small_cells)))
        if not self.h:
            raise ValueError("fmm create failed (bad kernel or config)")

    def tree(self, which):
        """Cells in pre-order: dict of level, index, center, hw, n_idx, n_children, indices."""
        pre = "fmm_" if self.L.prefix == "ref_" else ""
        f = self.L.fn(pre + "tree_cells", _L, [_P, _I, _P, _P, _P, _P, _P, _P])
        n = f(self.h, which, None, None, None, None, None, None)
        out = {k: np.zeros(n, dtype=np.int64) for k in ("level", "index", "n_idx", "n_children")}
        out["center"] = np.zeros((n, 3))
        out["hw"] = np.zeros((n, 3))
        f(self.h, which, _ptr(out["level"]), _ptr(out["index"]), _ptr(out["center"]),
          _ptr(out["hw"]), _ptr(out["n_idx"]), _ptr(out["n_children"]))
        g = self.L.fn(pre + "tree_indices", _L, [_P, _I, _P])
        m = g(self.h, which, None)
        idx = np.zeros(m, dtype=np.int64)
        g(self.h, which, _ptr(idx))
        out["indices"] = np.split(idx, np.cumsum(out["n_idx"])[:-1])
        return out

    def list(self, kind):
        pre = "fmm_" if self.L.prefix == "ref_" else ""
        f = self.L.fn(pre + "list", _L, [_P, _I, _P, _P])
        k = LISTS.index(kind) if isinstance(kind, str) else int(kind)
        n = f(self.h, k, None, None)
        a = np.zeros(n, dtype=np.int64)
        b = np.zeros(n, dtype=np.int64)
        f(self.h, k, _ptr(a), _ptr(b))
        return a, b

    def n_surf(self):
        pre = "fmm_" if self.L.prefix == "ref_" else ""
        return self.L.fn(pre + "n_surf", _L, [_P])(self.h)


class OracleFMM(_FMMBase):
    """The oracle restatement of FMMOperator<dim,R,C> (cpp/fmm.h:131-237).

    kernel: an id, or a name resolved in 2D when the points are [n][2]."""

    def __init__(self, kernel, obs_locs, obs_normals, src_locs, src_normals, src_weights,
                 mac, order, min_pts, d=0.05, small_cells=False, mu=1.0, nu=0.25):
        self._setup(_lib(), kernel, obs_locs, obs_normals, src_locs, src_normals,
                    src_weights, mac, order, min_pts, d, small_cells, mu, nu)
        L = self.L
        nlev = L.fn("n_levels", _L, [_P, _I])
        sysf = L.fn("c2e_system", _L, [_P, _I, _L, _P])
        setf = L.fn("set_c2e", _L, [_P, _I, _L, _P])
        n = self.n_surf() * self.R
        self.c2e = {0: [], 1: []}
        for which in (0, 1):
            for lev in range(nlev(self.h, which)):
                A = np.zeros((n, n))
                sysf(self.h, which, lev, _ptr(A))
                P = pinv_reference(A)
                self.c2e[which].append(P)
                setf(self.h, which, lev, _ptr(P))
        self._apply = L.fn("apply", None, [_P, _P, _P, _I, _D])

    def c2e_system(self, which, level):
        """The (R n_s) x (C n_s) system whose pseudo-inverse is the operator."""
        n = self.n_surf() * self.R
        A = np.zeros((n, n))
        self.L.fn("c2e_system", _L, [_P, _I, _L, _P])(self.h, which, level, _ptr(A))
        return A

    def ulp_floor(self, x, seed=0):
        """Relative change of this apply when every check-to-equivalent system
        is perturbed by one ulp (relative 2^-52 of each entry, random sign)
        before its pseudo-inverse: the agreement two correct FP64 evaluations
        of the plain form can be expected to reach (its pseudo-inverses keep
        singular values down to 1e-10 of the largest)."""
        y0 = self.apply(x)
        saved = {w: list(self.c2e[w]) for w in (0, 1)}
        rng = np.random.default_rng(seed)
        for which in (0, 1):
            for lev in range(len(saved[which])):
                A = self.c2e_system(which, lev)
                A = A * (1 + 2.0 ** -52 * rng.choice([-1.0, 1.0], size=A.shape))
                self.set_c2e(which, lev, pinv_reference(A))
        y1 = self.apply(x)
        for which in (0, 1):
            for lev, op in enumerate(saved[which]):
                self.set_c2e(which, lev, op)
        return float(np.linalg.norm(y1 - y0) / max(np.linalg.norm(y0), 1e-300))

    def set_c2e(self, which, level, op):
        """Install a check-to-equivalent operator (e.g. the reference's own)."""
        op = _f64(op)
        self.c2e[which][level] = op
        self.L.fn("set_c2e", _L, [_P, _I, _L, _P])(self.h, which, level, _ptr(op))

    def apply(self, x, mask=0xff, list_fraction=1.0):
        x = _f64(x)
        assert x.shape == (self.R * self.n_src,)
        y = np.zeros(self.R * self.n_obs)
        self._apply(self.h, _ptr(x), _ptr(y), int(mask), float(list_fraction))
        return y

    def __del__(self):
        if getattr(self, "h", None):
            self.L.fn("destroy", None, [_P])(self.h)
            self.h = None


class RefFMM(_FMMBase):
    """The reference FMMOperator itself, built from its sources (oracle/_ref)."""

    def __init__(self, kernel, obs_locs, obs_normals, src_locs, src_normals, src_weights,
                 mac, order, min_pts, d=0.05, small_cells=False, mu=1.0, nu=0.25):
        if "ref" not in _Lib._cache:
            _Lib._cache["ref"] = _Lib(REF_LIB_PATH, "ref_")
        self._setup(_Lib._cache["ref"], kernel, obs_locs, obs_normals, src_locs,
                    src_normals, src_weights, mac, order, min_pts, d, small_cells, mu, nu)

    def apply(self, x, mask=0xff):
        x = _f64(x)
        y = np.zeros(self.R * self.n_obs)
        self.L.fn("fmm_apply_masked", None, [_P, _I, _P, _P])(self.h, int(mask), _ptr(x), _ptr(y))
        return y

    def c2e(self, which, level):
        f = self.L.fn("fmm_c2e", _L, [_P, _I, _L, _P])
        n = self.n_surf() * self.R
        A = np.zeros((n, n))
        f(self.h, which, level, _ptr(A))
        return A

    def n_levels(self, which):
        return self.L.fn("fmm_c2e", _L, [_P, _I, _L, _P])(self.h, which, -1, None)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.fn("fmm_destroy", None, [_P])(self.h)
            self.h = None


def ref_available():
    return os.path.exists(REF_LIB_PATH)


def direct(kernel, obs_locs, obs_normals, src_locs, src_normals, src_weights, x,
           mu=1.0, nu=0.25):
    """FP64 direct N-body sum (the reference's nbody_eval over all pairs)."""
    dim = np.asarray(obs_locs).reshape(len(obs_locs), -1).shape[1] if len(obs_locs) else 3
    k = kernel_id(kernel, dim)
    R = kernel_components(k)
    ol, on = _pts3(obs_locs), _pts3(obs_normals)
    sl, sn, sw = _pts3(src_locs), _pts3(src_normals), _f64(src_weights)
    x = _f64(x)
    y = np.zeros(R * len(ol))
    f = _lib().fn("direct", _I, [_I, _D, _D, _P, _P, _L, _P, _P, _P, _L, _P, _P])
    f(k, mu, nu, _ptr(ol), _ptr(on), len(ol), _ptr(sl), _ptr(sn), _ptr(sw), len(sl),
      _ptr(x), _ptr(y))
    return y


def kernel_tensor(kernel, obs, src, nobs, nsrc, mu=1.0, nu=0.25, lib="oracle"):
    """One kernel tensor K(obs, src, nobs, nsrc) as an R x C array."""
    k = kernel_id(kernel, len(obs))
    L = _lib() if lib == "oracle" else _Lib._cache.setdefault("ref", _Lib(REF_LIB_PATH, "ref_"))
    f = L.fn("kernel", _I, [_I, _D, _D, _P, _P, _P, _P, _P])
    out = np.zeros(9)
    args = [_pts3(np.reshape(a, (1, -1)))[0] for a in (obs, src, nobs, nsrc)]
    n = f(k, mu, nu, *[_ptr(a) for a in args], _ptr(out))
    R = {9: 3, 4: 2}.get(n, 1)
    return out[:n].reshape(R, R)


def surface(order, dim=3, lib="oracle"):
    """Unit translation-surface points, [n][3] (z = 0 in 2D)."""
    L = _lib() if lib == "oracle" else _Lib._cache.setdefault("ref", _Lib(REF_LIB_PATH, "ref_"))
    f = L.fn("surface", _L, [_L, _I, _P])
    n = f(int(order), int(dim), None)
    p = np.zeros((n, 3))
    f(int(order), int(dim), _ptr(p))
    return p


def max_threads():
    return _lib().fn("max_threads", _I, [])()


# ---- the reference's nearfield construction (oracle/ref/nearfield_shim.cpp)

def _ref():
    return _Lib._cache.setdefault("ref", _Lib(REF_LIB_PATH, "ref_"))


def _mesh_args(vertices, facets):
    v = _pts3(vertices)
    f = np.ascontiguousarray(facets, dtype=np.int64)
    return v, f


def ref_nearfield(kernel, vertices, facets, strategy="sinh", near_tol=1e-4, sinh_order=5,
                  obs_near_order=2, obs_far_order=2, src_far_order=2, n_singular_steps=8,
                  far_threshold=3.0, which=0, mu=1.0, nu=0.25):
    """The reference's nearfield (which 0) or farfield-correction (which 1)
    CSR matrix of a mesh against itself: (n_rows, n_cols, values, cols, rowptr)."""
    dim = np.asarray(vertices).shape[1]
    k = kernel_id(kernel, dim)
    v, f = _mesh_args(vertices, facets)
    fn = _ref().fn("nearfield", _L, [_I, _D, _D, _I, _P, _L, _P, _L, _I, _D, _L, _L, _L, _L, _L,
                                     _D, _I, _P, _P, _P, _P, _L])
    shape = np.zeros(2, dtype=np.int64)
    args = [k, mu, nu, dim, _ptr(v), len(v), _ptr(f), len(f), 0 if strategy == "adaptive" else 1,
            near_tol, sinh_order, obs_near_order, obs_far_order, src_far_order, n_singular_steps,
            far_threshold, which, _ptr(shape)]
    nnz = fn(*args, None, None, None, 0)
    if nnz < 0:
        raise ValueError("reference nearfield failed")
    vals = np.zeros(nnz)
    cols = np.zeros(nnz, dtype=np.int64)
    rows = np.zeros(shape[0] + 1, dtype=np.int64)
    fn(*args, _ptr(vals), _ptr(cols), _ptr(rows), nnz)
    return int(shape[0]), int(shape[1]), vals, cols, rows


def ref_obs_points(vertices, facets, order):
    """The reference's Galerkin observation points: (locs, normals, dirs) [n][3]."""
    dim = np.asarray(vertices).shape[1]
    v, f = _mesh_args(vertices, facets)
    fn = _ref().fn("obs_points", _L, [_I, _P, _L, _P, _L, _L, _P, _P, _P])
    n = fn(dim, _ptr(v), len(v), _ptr(f), len(f), order, None, None, None)
    out = [np.zeros((n, 3)) for _ in range(3)]
    fn(dim, _ptr(v), len(v), _ptr(f), len(f), order, *[_ptr(a) for a in out])
    return tuple(out)


def ref_gauss_facet(dim, n):
    fn = _ref().fn("gauss_facet", _L, [_I, _L, _P, _P])
    k = fn(dim, n, None, None)
    x = np.zeros((k, dim - 1))
    w = np.zeros(k)
    fn(dim, n, _ptr(x), _ptr(w))
    return x, w


def ref_term(kernel, loc, normal, direction, facet, strategy="sinh", near_tol=1e-4, sinh_order=5,
             obs_near_order=2, obs_far_order=2, src_far_order=2, n_singular_steps=8,
             far_threshold=3.0, mu=1.0, nu=0.25):
    """One compute_term of the reference: [dim][R][C]."""
    dim = len(loc)
    k = kernel_id(kernel, dim)
    R = kernel_components(k)
    fn = _ref().fn("term", _L, [_I, _D, _D, _I, _D, _L, _L, _L, _L, _L, _D, _P, _P, _P, _P, _P])
    vec = [_pts3(np.reshape(a, (1, -1)))[0] for a in (loc, normal, direction)]
    fac = _pts3(np.reshape(facet, (dim, -1)))
    out = np.zeros(dim * R * R)
    fn(k, mu, nu, 0 if strategy == "adaptive" else 1, near_tol, sinh_order, obs_near_order,
       obs_far_order, src_far_order, n_singular_steps, far_threshold, *[_ptr(a) for a in vec],
       _ptr(fac), _ptr(out))
    return out.reshape(dim, R, R)


def ref_galerkin_interp(which, vertices, facets, n_components, order):
    """The reference's Galerkin (which 0) or interpolation (which 1) CSR
    operator: (n_rows, n_cols, values, cols, rowptr)."""
    dim = np.asarray(vertices).shape[1]
    v, f = _mesh_args(vertices, facets)
    fn = _ref().fn("galerkin_interp", _L, [_I, _I, _L, _P, _L, _P, _L, _L, _P, _P, _P, _P, _L])
    shape = np.zeros(2, dtype=np.int64)
    args = [which, dim, n_components, _ptr(v), len(v), _ptr(f), len(f), order, _ptr(shape)]
    nnz = fn(*args, None, None, None, 0)
    vals = np.zeros(nnz)
    cols = np.zeros(nnz, dtype=np.int64)
    rows = np.zeros(shape[0] + 1, dtype=np.int64)
    fn(*args, _ptr(vals), _ptr(cols), _ptr(rows), nnz)
    return int(shape[0]), int(shape[1]), vals, cols, rows


def ref_interior_dirs(locs, vertices, facets):
    """The reference's interior_obs_pts limit directions, [n][3]."""
    dim = np.asarray(vertices).shape[1]
    v, f = _mesh_args(vertices, facets)
    l = _pts3(locs)
    fn = _ref().fn("interior_dirs", _L, [_I, _P, _L, _P, _L, _P, _L, _P])
    out = np.zeros((len(l), 3))
    fn(dim, _ptr(l), len(l), _ptr(v), len(v), _ptr(f), len(f), _ptr(out))
    return out


def ref_dense_interior(kernel, vertices, facets, locs, normals, sinh_order=5, obs_near_order=2,
                       obs_far_order=2, src_far_order=2, n_singular_steps=8, far_threshold=3.0,
                       mu=1.0, nu=0.25):
    """The reference's dense_interior_operator (sinh strategy) for given points
    against a mesh: the dense matrix [R n, C n_dofs]."""
    dim = np.asarray(vertices).shape[1]
    k = kernel_id(kernel, dim)
    v, f = _mesh_args(vertices, facets)
    l, n = _pts3(locs), _pts3(normals)
    fn = _ref().fn("dense_interior", _L, [_I, _D, _D, _I, _P, _L, _P, _L, _P, _P, _L, _L, _L, _L,
                                          _L, _L, _D, _P])
    args = [k, mu, nu, dim, _ptr(v), len(v), _ptr(f), len(f), _ptr(l), _ptr(n), len(l), sinh_order,
            obs_near_order, obs_far_order, src_far_order, n_singular_steps, far_threshold]
    cnt = fn(*args, None)
    if cnt < 0:
        raise ValueError("reference dense interior operator failed")
    out = np.zeros(cnt)
    fn(*args, _ptr(out))
    return out.reshape(kernel_components(k) * len(l), -1)


def ref_mass(vertices, facets, R, n_q):
    """The reference's mass_operator<dim,R,R>: (n_rows, n_cols, values, cols, rowptr)."""
    dim = np.asarray(vertices).shape[1]
    v, f = _mesh_args(vertices, facets)
    fn = _ref().fn("mass", _L, [_I, _L, _P, _L, _P, _L, _L, _P, _P, _P, _P, _L])
    shape = np.zeros(2, dtype=np.int64)
    args = [dim, R, _ptr(v), len(v), _ptr(f), len(f), n_q, _ptr(shape)]
    nnz = fn(*args, None, None, None, 0)
    vals = np.zeros(nnz)
    cols = np.zeros(nnz, dtype=np.int64)
    rows = np.zeros(shape[0] + 1, dtype=np.int64)
    fn(*args, _ptr(vals), _ptr(cols), _ptr(rows), nnz)
    return int(shape[0]), int(shape[1]), vals, cols, rows


def ref_nearfield_points(kernel, vertices, facets, locs, normals, sinh_order=5, obs_near_order=2,
                         obs_far_order=2, src_far_order=2, n_singular_steps=8, far_threshold=3.0,
                         which=0, mu=1.0, nu=0.25):
    """The reference's nearfield (which 0) / correction (1) CSR for given points."""
    dim = np.asarray(vertices).shape[1]
    k = kernel_id(kernel, dim)
    v, f = _mesh_args(vertices, facets)
    l, n = _pts3(locs), _pts3(normals)
    fn = _ref().fn("nearfield_points", _L, [_I, _D, _D, _I, _P, _L, _P, _L, _P, _P, _L, _L, _L, _L,
                                            _L, _L, _D, _I, _P, _P, _P, _P, _L])
    shape = np.zeros(2, dtype=np.int64)
    args = [k, mu, nu, dim, _ptr(v), len(v), _ptr(f), len(f), _ptr(l), _ptr(n), len(l), sinh_order,
            obs_near_order, obs_far_order, src_far_order, n_singular_steps, far_threshold, which,
            _ptr(shape)]
    nnz = fn(*args, None, None, None, 0)
    if nnz < 0:
        raise ValueError("reference nearfield failed")
    vals = np.zeros(nnz)
    cols = np.zeros(nnz, dtype=np.int64)
    rows = np.zeros(shape[0] + 1, dtype=np.int64)
    fn(*args, _ptr(vals), _ptr(cols), _ptr(rows), nnz)
    return int(shape[0]), int(shape[1]), vals, cols, rows


def ref_dense_boundary(kernel, vertices, facets, sinh_order=5, obs_near_order=2, obs_far_order=2,
                       src_far_order=2, n_singular_steps=8, far_threshold=3.0, mu=1.0, nu=0.25):
    """The reference's dense_boundary_operator (sinh strategy) of a mesh against
    itself: the dense matrix [R n_dofs, C n_dofs]."""
    dim = np.asarray(vertices).shape[1]
    k = kernel_id(kernel, dim)
    v, f = _mesh_args(vertices, facets)
    fn = _ref().fn("dense_boundary", _L, [_I, _D, _D, _I, _P, _L, _P, _L, _L, _L, _L, _L, _L, _D, _P])
    args = [k, mu, nu, dim, _ptr(v), len(v), _ptr(f), len(f), sinh_order, obs_near_order,
            obs_far_order, src_far_order, n_singular_steps, far_threshold]
    n = fn(*args, None)
    out = np.zeros(n)
    fn(*args, _ptr(out))
    R = kernel_components(k)
    rows = R * dim * len(f)
    return out.reshape(rows, -1)
