"""3D operators with the reference's Python names (tbempy.ThreeD).

Mirrors the hot-path part of the reference binding: ``FMMConfig(mac, order,
min_pts_per_cell, d, account_for_small_cells)`` (python_wrapper/fmm_config.cpp:7),
the kernel classes (python_wrapper/kernels.cpp:11-27) and operators with
``apply / n_rows / n_cols / clone`` (python_wrapper/op_wrap.h:4-11), plus the
C++-only ``FMMOperator(K, NBodyData, FMMConfig)`` (cpp/fmm.h:146-147) that
the reference never exposed, ``SparseOperator`` (python_wrapper/linalg.cpp)
and ``IntegralOperator`` (cpp/integral_operator.h:26-64).

``apply`` accepts numpy arrays (host; copied in and out inside the call) or
float64 torch tensors (device, no copies); several right-hand sides are
passed as a 2-D array [n_rhs, n_cols].  Everything runs through the C ABI
of lib/libtbem_gpu.so.
"""
import ctypes as C

import numpy as np

from . import _lib as _L
from ._lib import check

try:  # torch is optional: plumbing for device tensors only
    import torch
except Exception:  # pragma: no cover
    torch = None


class FMMConfig:
    """FMMConfig (cpp/fmm.h:73-96); ``order`` = requested surface points."""

    def __init__(self, mac, order, min_pts_per_cell, d, account_for_small_cells):
        self.mac = float(mac)
        self.order = int(order)
        self.min_pts_per_cell = int(min_pts_per_cell)
        self.d = float(d)
        self.account_for_small_cells = bool(account_for_small_cells)

    def _c(self):
        return _L.TbemFmmConfig(self.mac, self.order, self.min_pts_per_cell, self.d,
                                int(self.account_for_small_cells))

    def __repr__(self):
        return ("FMMConfig(mac=%g, order=%d, min_pts_per_cell=%d, d=%g, "
                "account_for_small_cells=%s)" % (self.mac, self.order, self.min_pts_per_cell,
                                                 self.d, self.account_for_small_cells))


class Kernel:
    kernel_id = -1
    tensor_dim = 1
    space_dim = 3

    def params(self):
        return None


class LaplaceSingle(Kernel):
    """1 / (4 pi r) (cpp/laplace_kernels.h:19-32)."""
    kernel_id = 0


class LaplaceDouble(Kernel):
    """n_src . (y - x) / (4 pi r^3) (cpp/laplace_kernels.h:35-48)."""
    kernel_id = 1


class IdentityScalar(Kernel):
    """Identity test kernel (cpp/identity_kernels.h:9-40)."""
    kernel_id = 5


class _Elastic(Kernel):
    tensor_dim = 3

    def __init__(self, shear_modulus, poisson_ratio):
        self.shear_modulus = float(shear_modulus)
        self.poisson_ratio = float(poisson_ratio)

    def params(self):
        return np.array([self.shear_modulus, self.poisson_ratio], dtype=np.float64)


class ElasticDisplacement(_Elastic):
    """Kelvin displacement kernel (cpp/elastic_kernels.h:192-227)."""
    kernel_id = 2


class ElasticTraction(_Elastic):
    """Kelvin traction kernel (cpp/elastic_kernels.h:230-269)."""
    kernel_id = 3


class ElasticAdjointTraction(_Elastic):
    """Adjoint traction kernel (cpp/elastic_kernels.h:272-311)."""
    kernel_id = 4


class ElasticHypersingular(_Elastic):
    """Hypersingular kernel: traction of the displacement of a dislocation
    (cpp/elastic_kernels.h:314-365)."""
    kernel_id = 6


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def _ptr(a):
    if a is None:
        return None
    if torch is not None and isinstance(a, torch.Tensor):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


def _stream_of(t):
    if torch is not None and isinstance(t, torch.Tensor) and t.is_cuda:
        h = torch.cuda.current_stream(t.device).cuda_stream
        # torch's default stream is the legacy stream (handle 0); NULL means
        # "the operator's own stream" in the C ABI, so name it explicitly
        return C.c_void_p(h if h else 1)
    return None


def _prep_in(x, n_cols):
    """-> (buffer, n_rhs, is_torch, squeeze)"""
    if torch is not None and isinstance(x, torch.Tensor):
        if x.dtype != torch.float64:
            raise TypeError("operator inputs are float64")
        squeeze = x.dim() == 1
        xx = x.reshape(-1, n_cols).contiguous()
        return xx, xx.shape[0], True, squeeze
    x = np.asarray(x, dtype=np.float64)
    squeeze = x.ndim == 1
    if n_cols == 0:
        xx = np.zeros((1 if squeeze else max(x.shape[0], 1), 0))
        return xx, xx.shape[0], False, squeeze
    xx = np.ascontiguousarray(x.reshape(-1, n_cols))
    return xx, xx.shape[0], False, squeeze


def _alloc_out(like, is_torch, n_rhs, n_rows):
    if is_torch:
        return torch.empty((n_rhs, n_rows), dtype=torch.float64, device=like.device)
    return np.empty((n_rhs, n_rows), dtype=np.float64)


class OperatorI:
    """The reference operator interface (cpp/operator.h:14-19)."""

    def n_rows(self):
        raise NotImplementedError

    def n_cols(self):
        raise NotImplementedError

    def apply(self, x):
        raise NotImplementedError

    def clone(self):
        raise NotImplementedError


class FMMOperator(OperatorI):
    """KIFMM operator (cpp/fmm.h:131-237) on the GPU.

    precision: "fp64" (plain form: the reference's surfaces and formulation),
    "mixed" (precision form: pre-combined operators applied with FP32 /
    tensor-core arithmetic, FP32 P2P with compensated sums) or
    "fp64_compressed" (the precision form's operators applied in FP64:
    linear to rounding, the O(N) residual operator of iterative refinement).
    """

    def __init__(self, K, obs_locs, obs_normals, src_locs, src_normals, src_weights, config,
                 precision="fp64", device=0, svd_threshold=1e-10, host_only=False,
                 m2l_path=0, m2l_rank_tol=1e-7, p2p_block=0, p2m_block=0, tc_shape=0,
                 _handle=None):
        self.K = K
        self.config = config
        self.precision = precision
        self.R = K.tensor_dim
        if _handle is not None:
            self._h = _handle
            return
        dim = K.space_dim
        self._obs_locs = _f64(obs_locs, (-1, dim))
        self._obs_normals = _f64(obs_normals, (-1, dim))
        self._src_locs = _f64(src_locs, (-1, dim))
        self._src_normals = _f64(src_normals, (-1, dim))
        self._src_weights = _f64(src_weights, (-1,))
        opt = _L.TbemGpuOptions()
        _L.lib().tbem_default_options(C.byref(opt))
        opt.precision = _L.PRECISION[precision]
        opt.device = int(device)
        opt.svd_threshold = float(svd_threshold)
        opt.host_only = int(bool(host_only))
        opt.m2l_path = int(m2l_path)
        opt.m2l_rank_tol = float(m2l_rank_tol)
        opt.p2p_block = int(p2p_block)
        opt.p2m_block = int(p2m_block)
        opt.tc_shape = int(tc_shape)
        cfg = config._c()
        h = C.c_void_p()
        params = K.params()
        check(_L.lib().tbem_fmm_create(
            K.kernel_id, _ptr(params), _ptr(self._obs_locs), _ptr(self._obs_normals),
            len(self._obs_locs), _ptr(self._src_locs), _ptr(self._src_normals),
            _ptr(self._src_weights), len(self._src_locs), C.byref(cfg), C.byref(opt),
            C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _L._lib is not None:
            _L._lib.tbem_fmm_destroy(h)
            self._h = None

    def n_rows(self):
        return check(_L.lib().tbem_fmm_n_rows(self._h))

    def n_cols(self):
        return check(_L.lib().tbem_fmm_n_cols(self._h))

    def _run(self, fn, x, n_in, n_out):
        xx, n_rhs, is_t, squeeze = _prep_in(x, n_in)
        y = _alloc_out(xx, is_t, n_rhs, n_out)
        check(fn(self._h, _ptr(xx), _ptr(y), int(n_rhs), _stream_of(xx)))
        return y.reshape(-1) if squeeze else y

    def apply(self, x):
        """y = A x (FMMOperator::apply, cpp/fmm.cpp:551-557)."""
        return self._run(_L.lib().tbem_fmm_apply, x, self.n_cols(), self.n_rows())

    def apply_adjoint(self, z):
        """w = A^T z (the FMM passes transposed, in reverse order)."""
        return self._run(_L.lib().tbem_fmm_apply_adjoint, z, self.n_rows(), self.n_cols())

    def source_gradients(self, x, r):
        """Derivatives of L = r^T A x (one right-hand side) with respect to
        the source points' positions, normals and weights, through the FMM
        (the compressed forms): a dict keyed src_locs [n_src, 3],
        src_normals [n_src, 3], src_weights [n_src], numpy or float64 CUDA
        tensors like x."""
        is_t = torch is not None and isinstance(x, torch.Tensor)
        n = self.n_cols() // self.K.tensor_dim
        if is_t:
            xx, rr = x.reshape(-1).contiguous(), r.reshape(-1).contiguous()
            out = {k: torch.empty(s, dtype=torch.float64, device=xx.device)
                   for k, s in (("src_locs", (n, 3)), ("src_normals", (n, 3)), ("src_weights", (n,)))}
        else:
            xx, rr = _f64(x, (-1,)), _f64(r, (-1,))
            out = {"src_locs": np.empty((n, 3)), "src_normals": np.empty((n, 3)),
                   "src_weights": np.empty(n)}
        if xx.shape[0] != self.n_cols() or rr.shape[0] != self.n_rows():
            raise ValueError("x has n_cols and r n_rows entries (one right-hand side)")
        check(_L.lib().tbem_fmm_source_gradients(
            self._h, _ptr(xx), _ptr(rr), _ptr(out["src_locs"]), _ptr(out["src_normals"]),
            _ptr(out["src_weights"]), _stream_of(xx)))
        return out

    def observation_gradients(self, x, r):
        """Derivatives of L = r^T A x (one right-hand side) with respect to
        the observation points' positions and normals, through the FMM (the
        compressed forms): a dict keyed obs_locs [n_obs, 3] and obs_normals
        [n_obs, 3], numpy or float64 CUDA tensors like x."""
        is_t = torch is not None and isinstance(x, torch.Tensor)
        n = self.n_rows() // self.K.tensor_dim
        if is_t:
            xx, rr = x.reshape(-1).contiguous(), r.reshape(-1).contiguous()
            out = {k: torch.empty((n, 3), dtype=torch.float64, device=xx.device)
                   for k in ("obs_locs", "obs_normals")}
        else:
            xx, rr = _f64(x, (-1,)), _f64(r, (-1,))
            out = {"obs_locs": np.empty((n, 3)), "obs_normals": np.empty((n, 3))}
        if xx.shape[0] != self.n_cols() or rr.shape[0] != self.n_rows():
            raise ValueError("x has n_cols and r n_rows entries (one right-hand side)")
        check(_L.lib().tbem_fmm_observation_gradients(
            self._h, _ptr(xx), _ptr(rr), _ptr(out["obs_locs"]), _ptr(out["obs_normals"]),
            _stream_of(xx)))
        return out

    def clone(self):
        h = C.c_void_p()
        check(_L.lib().tbem_fmm_clone(self._h, C.byref(h)))
        return FMMOperator(self.K, None, None, None, None, None, self.config,
                           precision=self.precision, _handle=h)

    # -- introspection ---------------------------------------------------------
    def n_surface(self):
        return check(_L.lib().tbem_fmm_n_surface(self._h))

    def tree(self, which):
        """Cells in pre-order (which: 0 source tree, 1 observation tree);
        centers and half widths are [n][3] (z = 0 for a 2D operator)."""
        f = _L.lib().tbem_fmm_tree_cells
        n = check(f(self._h, which, None, None, None, None, None, None))
        out = {k: np.zeros(n, dtype=np.int64) for k in ("level", "index", "n_idx", "n_children")}
        out["center"] = np.zeros((n, 3))
        out["hw"] = np.zeros((n, 3))
        check(f(self._h, which, _ptr(out["level"]), _ptr(out["index"]), _ptr(out["center"]),
                _ptr(out["hw"]), _ptr(out["n_idx"]), _ptr(out["n_children"])))
        g = _L.lib().tbem_fmm_tree_indices
        m = check(g(self._h, which, None))
        idx = np.zeros(m, dtype=np.int64)
        check(g(self._h, which, _ptr(idx)))
        out["indices"] = np.split(idx, np.cumsum(out["n_idx"])[:-1])
        return out

    def list(self, kind):
        from_name = ["p2m", "m2m", "p2p", "m2p", "p2l", "m2l", "l2l", "l2p"]
        k = from_name.index(kind) if isinstance(kind, str) else int(kind)
        f = _L.lib().tbem_fmm_list
        n = check(f(self._h, k, None, None))
        a = np.zeros(n, dtype=np.int64)
        b = np.zeros(n, dtype=np.int64)
        check(f(self._h, k, _ptr(a), _ptr(b)))
        return a, b

    def n_c2e_levels(self, which):
        return check(_L.lib().tbem_fmm_n_c2e_levels(self._h, which))

    def get_c2e(self, which, level):
        n = self.n_surface() * self.R
        out = np.zeros((n, n))
        check(_L.lib().tbem_fmm_get_c2e(self._h, which, level, _ptr(out)))
        return out

    def set_c2e(self, which, level, op):
        op = _f64(op)
        check(_L.lib().tbem_fmm_set_c2e(self._h, which, level, _ptr(op)))

    def set_timing(self, enabled=True):
        check(_L.lib().tbem_fmm_set_timing(self._h, int(bool(enabled))))

    def p2p_block(self):
        """Threads per target of the point-to-point pass (autotuned)."""
        return check(_L.lib().tbem_fmm_p2p_block(self._h))

    def tc_tile(self):
        """N tile of the tensor-core translations (autotuned; 0 if unused)."""
        return check(_L.lib().tbem_fmm_tc_tile(self._h))

    def m2l_ranks(self):
        """(r_in, r_out) of the SVD-compressed M2L; (0, 0) when uncompressed."""
        a, b = C.c_long(), C.c_long()
        check(_L.lib().tbem_fmm_m2l_ranks(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def last_launches(self):
        """Kernel launches made by the last apply."""
        return check(_L.lib().tbem_fmm_last_launches(self._h))

    def sync(self, stream=None):
        """Wait for this operator's device work; raises TbemError (code -5)
        if a tensor-core pass of an earlier apply gave up waiting.  An apply
        into device memory is asynchronous, so such a failure would otherwise
        only surface on the next apply."""
        check(_L.lib().tbem_fmm_sync(self._h, stream))

    def set_wait_cycles(self, cycles):
        """Budget (SM cycles) of the tensor-core kernels' bounded waits;
        0 restores the default (about two seconds).  For tests of the
        timeout path."""
        check(_L.lib().tbem_fmm_set_wait_cycles(self._h, int(cycles)))

    def phase_times(self):
        cap = 32
        names = (C.c_char_p * cap)()
        ms = np.zeros(cap)
        k = check(_L.lib().tbem_fmm_phase_times(self._h, names, _ptr(ms), cap))
        return [(names[i].decode(), float(ms[i])) for i in range(min(k, cap))]

    def setup_times(self):
        """Wall seconds of the construction phases, [(name, seconds)]."""
        cap = 16
        names = (C.c_char_p * cap)()
        s = np.zeros(cap)
        k = check(_L.lib().tbem_fmm_setup_times(self._h, names, _ptr(s), cap))
        return [(names[i].decode(), float(s[i])) for i in range(min(k, cap))]


class BatchedFMMOperator(FMMOperator):
    """One operator over many independent meshes (the batched form; the
    reference builds one FMMOperator per mesh).  ``offsets[m]:offsets[m+1]``
    are mesh m's rows of ``locs`` / ``normals`` / ``weights``; within a mesh
    the observation points are its source points.  Applies take
    x[rhs][C][N] over all N points (meshes concatenated) and return
    y[rhs][R][N]; every pass covers all meshes in one launch."""

    def __init__(self, K, locs, normals, weights, offsets, config, precision="mixed", device=0,
                 svd_threshold=1e-10, host_only=False, m2l_path=0, m2l_rank_tol=1e-7,
                 p2p_block=0, p2m_block=0, tc_shape=0, _handle=None):
        self.K = K
        self.config = config
        self.precision = precision
        self.R = K.tensor_dim
        if _handle is not None:
            self._h = _handle
            return
        self._locs = _f64(locs, (-1, 3))
        self._normals = _f64(normals, (-1, 3))
        self._weights = _f64(weights, (-1,))
        self.offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        opt = _L.TbemGpuOptions()
        _L.lib().tbem_default_options(C.byref(opt))
        opt.precision = _L.PRECISION[precision]
        opt.device = int(device)
        opt.svd_threshold = float(svd_threshold)
        opt.host_only = int(bool(host_only))
        opt.m2l_path = int(m2l_path)
        opt.m2l_rank_tol = float(m2l_rank_tol)
        opt.p2p_block = int(p2p_block)
        opt.p2m_block = int(p2m_block)
        opt.tc_shape = int(tc_shape)
        cfg = config._c()
        h = C.c_void_p()
        check(_L.lib().tbem_fmm_batch_create(
            K.kernel_id, _ptr(K.params()), len(self.offsets) - 1, _ptr(self.offsets),
            _ptr(self._locs), _ptr(self._normals), _ptr(self._weights), C.byref(cfg),
            C.byref(opt), C.byref(h)))
        self._h = h

    def n_meshes(self):
        return check(_L.lib().tbem_fmm_n_meshes(self._h))

    def clone(self):
        h = C.c_void_p()
        check(_L.lib().tbem_fmm_clone(self._h, C.byref(h)))
        return BatchedFMMOperator(self.K, None, None, None, None, self.config,
                                  precision=self.precision, _handle=h)


class FMMGraph:
    """One CUDA graph replaying the applies of several operators (e.g. one per
    mesh of a batch) between fixed float64 CUDA tensors (tbem_fmm_graph_*).

    ops: FMMOperators; xs / ys: CUDA tensors, [n_cols] / [n_rows] (or
    [n_rhs, n] with n_rhs given).  Building runs each apply once (writing ys).
    launch() replays all of them with one graph launch (asynchronous; the
    results are in ys after a device synchronization)."""

    def __init__(self, ops, xs, ys, n_rhs=1, adjoint=False):
        self.ops, self.xs, self.ys = list(ops), list(xs), list(ys)  # keep alive
        n = len(self.ops)
        handles = (C.c_void_p * n)(*[op._h.value if hasattr(op._h, "value") else op._h
                                     for op in self.ops])
        xp = (C.c_void_p * n)(*[t.data_ptr() for t in self.xs])
        yp = (C.c_void_p * n)(*[t.data_ptr() for t in self.ys])
        h = C.c_void_p()
        check(_L.lib().tbem_fmm_graph_create(handles, n, xp, yp, int(n_rhs), int(bool(adjoint)),
                                             C.byref(h)))
        self._h = h

    def launch(self, stream=None):
        check(_L.lib().tbem_fmm_graph_launch(self._h, stream))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _L._lib is not None:
            _L._lib.tbem_fmm_graph_destroy(h)
            self._h = None


class DirectOperator(OperatorI):
    """FP64 direct N-body operator on the GPU (make_direct_nbody_operator,
    cpp/nbody_operator.h:143-152, applied matrix-free like nbody_eval)."""

    def __init__(self, K, obs_locs, obs_normals, src_locs, src_normals, src_weights):
        self.K = K
        self.R = K.tensor_dim
        dim = K.space_dim
        self._obs_locs = _f64(obs_locs, (-1, dim))
        self._obs_normals = _f64(obs_normals, (-1, dim))
        self._src_locs = _f64(src_locs, (-1, dim))
        self._src_normals = _f64(src_normals, (-1, dim))
        self._src_weights = _f64(src_weights, (-1,))
        self._params = K.params()

    def n_rows(self):
        return self.R * len(self._obs_locs)

    def n_cols(self):
        return self.R * len(self._src_locs)

    def apply(self, x):
        xx, n_rhs, is_t, squeeze = _prep_in(x, self.n_cols())
        y = _alloc_out(xx, is_t, n_rhs, self.n_rows())
        check(_L.lib().tbem_direct_apply(
            self.K.kernel_id, _ptr(self._params), _ptr(self._obs_locs), _ptr(self._obs_normals),
            len(self._obs_locs), _ptr(self._src_locs), _ptr(self._src_normals),
            _ptr(self._src_weights), len(self._src_locs), _ptr(xx), _ptr(y), int(n_rhs),
            _stream_of(xx)))
        return y.reshape(-1) if squeeze else y

    def clone(self):
        return DirectOperator(self.K, self._obs_locs, self._obs_normals, self._src_locs,
                              self._src_normals, self._src_weights)


def clear_setup_cache():
    """Empty the process's setup cache (the pseudo-inverses and M2L
    eigenbases later constructions with the same kernel parameters and cell
    geometry reuse)."""
    check(_L.lib().tbem_setup_cache_clear())


def fma_peak_tflops(fp64=False, device=0):
    """The device's measured FMA rate (TFLOP/s, FMA = 2 flops) from the
    library's microbenchmark: the denominator of the evaluation kernels'
    roofline."""
    out = np.zeros(1)
    check(_L.lib().tbem_fma_peak(int(device), int(bool(fp64)), _ptr(out)))
    return float(out[0])


def direct_gradients(K, obs_locs, obs_normals, src_locs, src_normals, src_weights, x, r):
    """Kernel-gradient pass: derivatives of L = r^T A x (A the direct
    operator) with respect to every point position, normal and weight and to
    x.  Arrays may be numpy (host) or float64 CUDA tensors; returns the same
    kind, keyed obs_locs, obs_normals, src_locs, src_normals, src_weights, x."""
    if K.space_dim != 3:
        raise ValueError("the kernel-gradient pass takes the 3D kernels")
    is_t = torch is not None and isinstance(obs_locs, torch.Tensor)

    def prep(a, shape):
        if is_t:
            return a.reshape(shape).contiguous()
        return _f64(a, shape)

    ol, on = prep(obs_locs, (-1, 3)), prep(obs_normals, (-1, 3))
    sl, sn = prep(src_locs, (-1, 3)), prep(src_normals, (-1, 3))
    sw = prep(src_weights, (-1,))
    xx, rr = prep(x, (-1,)), prep(r, (-1,))
    n_obs, n_src = ol.shape[0], sl.shape[0]

    def out(shape):
        if is_t:
            return torch.empty(shape, dtype=torch.float64, device=ol.device)
        return np.empty(shape)

    g = {"obs_locs": out((n_obs, 3)), "obs_normals": out((n_obs, 3)),
         "src_locs": out((n_src, 3)), "src_normals": out((n_src, 3)),
         "src_weights": out((n_src,)), "x": out((K.tensor_dim * n_src,))}
    check(_L.lib().tbem_direct_gradients(
        K.kernel_id, _ptr(K.params()), _ptr(ol), _ptr(on), n_obs, _ptr(sl), _ptr(sn), _ptr(sw),
        n_src, _ptr(xx), _ptr(rr), _ptr(g["obs_locs"]), _ptr(g["obs_normals"]),
        _ptr(g["src_locs"]), _ptr(g["src_normals"]), _ptr(g["src_weights"]), _ptr(g["x"]),
        _stream_of(ol)))
    return g


class DenseOperator(OperatorI):
    """A dense matrix operator (DenseOperator, cpp/dense_operator.h:11-40;
    python_wrapper/linalg.cpp:15-20): row-major data of n_rows x n_cols,
    ``data()`` the flat copy, applied on the GPU (through the CSR kernel, built
    on the first apply)."""

    def __init__(self, n_rows, n_cols, data):
        self._shape = (int(n_rows), int(n_cols))
        self._data = np.ascontiguousarray(data, dtype=np.float64).reshape(-1)
        if self._data.size != self._shape[0] * self._shape[1]:
            raise ValueError("data must hold n_rows * n_cols values")
        self._op = None

    def n_rows(self):
        return self._shape[0]

    def n_cols(self):
        return self._shape[1]

    def n_elements(self):
        return self._data.size

    def data(self):
        return self._data.copy()

    def to_dense(self):
        return self._data.reshape(self._shape).copy()

    def apply(self, x):
        if self._op is None:
            nr, nc = self._shape
            self._op = SparseOperator(nr, nc, self._data, np.tile(np.arange(nc, dtype=np.int64), nr),
                                      np.arange(nr + 1, dtype=np.int64) * nc)
        return self._op.apply(x)

    def clone(self):
        return DenseOperator(self._shape[0], self._shape[1], self._data)


class SparseOperator(OperatorI):
    """CSR operator (cpp/sparse_operator.h:44-83) with a GPU apply."""

    def __init__(self, n_rows, n_cols, values, column_indices, row_ptrs):
        self._shape = (int(n_rows), int(n_cols))
        self._values = _f64(values, (-1,))
        self._cols = np.ascontiguousarray(column_indices, dtype=np.int64)
        self._rows = np.ascontiguousarray(row_ptrs, dtype=np.int64)
        h = C.c_void_p()
        check(_L.lib().tbem_csr_create(self._shape[0], self._shape[1], _ptr(self._values),
                                       _ptr(self._cols), _ptr(self._rows), C.byref(h)))
        self._h = h

    @classmethod
    def _from_handle(cls, h):
        """Wrap a CSR operator the library built (its arrays read back once)."""
        self = cls.__new__(cls)
        L = _L.lib()
        nr, nc = C.c_long(), C.c_long()
        check(L.tbem_csr_shape(h, C.byref(nr), C.byref(nc)))
        nnz = check(L.tbem_csr_nnz(h))
        self._shape = (nr.value, nc.value)
        self._values = np.zeros(nnz)
        self._cols = np.zeros(nnz, dtype=np.int64)
        self._rows = np.zeros(nr.value + 1, dtype=np.int64)
        check(L.tbem_csr_download(h, _ptr(self._values), _ptr(self._cols), _ptr(self._rows)))
        self._h = h
        return self

    @staticmethod
    def csr_from_coo(n_rows, n_cols, rows, cols, values):
        """csr_from_coo (cpp/sparse_operator.cpp:140-172): entries keep their
        input order inside a row."""
        rows = np.asarray(rows, dtype=np.int64)
        cols = np.asarray(cols, dtype=np.int64)
        values = np.asarray(values, dtype=np.float64)
        order = np.argsort(rows, kind="stable")
        counts = np.bincount(rows, minlength=n_rows)
        row_ptrs = np.concatenate([[0], np.cumsum(counts)])
        return SparseOperator(n_rows, n_cols, values[order], cols[order], row_ptrs)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _L._lib is not None:
            _L._lib.tbem_csr_destroy(h)
            self._h = None

    def n_rows(self):
        return self._shape[0]

    def n_cols(self):
        return self._shape[1]

    def nnz(self):
        return check(_L.lib().tbem_csr_nnz(self._h))

    def values(self):
        return self._values.copy()

    def column_indices(self):
        return self._cols.copy()

    def row_ptrs(self):
        return self._rows.copy()

    def to_dense(self):
        d = np.zeros(self._shape)
        for i in range(self._shape[0]):
            for k in range(self._rows[i], self._rows[i + 1]):
                d[i, self._cols[k]] += self._values[k]
        return d

    def apply(self, x):
        xx, n_rhs, is_t, squeeze = _prep_in(x, self.n_cols())
        y = _alloc_out(xx, is_t, n_rhs, self.n_rows())
        check(_L.lib().tbem_csr_apply(self._h, _ptr(xx), _ptr(y), int(n_rhs), _stream_of(xx)))
        return y.reshape(-1) if squeeze else y

    def clone(self):
        return SparseOperator(self._shape[0], self._shape[1], self._values, self._cols,
                              self._rows)


class IntegralOperator(OperatorI):
    """A = G (F I) + N + C (cpp/integral_operator.h:13-63): galerkin,
    farfield (e.g. an FMMOperator), interpolation, nearfield and the
    farfield correction, all applied on the GPU.  With sparse operators and
    an FMMOperator farfield the chain runs on the device in one call
    (tbem_integral_apply); any other farfield (e.g. a DirectOperator) is
    composed step by step."""

    def __init__(self, nearfield, farfield_correction, galerkin, farfield, interp):
        self.nearfield = nearfield
        self.farfield_correction = farfield_correction
        self.galerkin = galerkin
        self.farfield = farfield
        self.interp = interp
        self._h = None
        if isinstance(farfield, FMMOperator) and all(
                isinstance(o, SparseOperator) for o in (nearfield, farfield_correction, galerkin, interp)):
            h = C.c_void_p()
            check(_L.lib().tbem_integral_create(nearfield._h, farfield_correction._h, galerkin._h,
                                                farfield._h, interp._h, C.byref(h)))
            self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _L._lib is not None:
            _L._lib.tbem_integral_destroy(h)
            self._h = None

    def n_rows(self):
        return self.galerkin.n_rows()

    def n_cols(self):
        return self.nearfield.n_cols()

    def apply(self, x):
        if self._h is not None:
            xx, n_rhs, is_t, squeeze = _prep_in(x, self.n_cols())
            y = _alloc_out(xx, is_t, n_rhs, self.n_rows())
            check(_L.lib().tbem_integral_apply(self._h, _ptr(xx), _ptr(y), int(n_rhs), _stream_of(xx)))
            return y.reshape(-1) if squeeze else y
        far = self.galerkin.apply(self.farfield.apply(self.interp.apply(x)))
        return self.nearfield.apply(x) + far + self.farfield_correction.apply(x)

    def clone(self):
        return IntegralOperator(self.nearfield.clone(), self.farfield_correction.clone(),
                                self.galerkin.clone(), self.farfield.clone(), self.interp.clone())


# boundary-operator assembly (nearfield / correction matrices on the GPU,
# Galerkin and interpolation operators, boundary_operator)
from .bem import (Mesh, IntegrationStrategy, boundary_operator, farfield_correction_operator,  # noqa: E402,F401
                  galerkin_csr, galerkin_obs_points, galerkin_operator, gauss_facet,
                  interpolation_csr, interpolation_operator, dense_interior_operator,
                  dense_boundary_operator,
                  interior_limit_directions, mass_csr, mass_operator_scalar, mass_operator_tensor,
                  make_adaptive_integrator, make_sinh_integrator, nearfield_operator,
                  quadrature_points)
