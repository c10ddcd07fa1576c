"""GMRES and FP64 iterative refinement around the operator apply.

The reference solves with scipy's GMRES on a LinearOperator whose matvec is
``op.apply`` (acceptance_tests/laplace.py:21-31).  Here:

* ``gmres(matvec, b, restart, tol, maxiter)`` -- restarted GMRES with modified
  Gram-Schmidt and Givens rotations, on numpy or torch vectors (whatever the
  matvec takes and returns);
* ``refined_solve(apply_fp64, apply_fast, b, tol)`` -- FP64 iterative
  refinement: the residual r = b - A x is formed with the FP64 operator, the
  correction A d = r is solved loosely with the fast (mixed-precision)
  operator, x += d, until ||r|| / ||b|| <= tol.  The fast operator's own error
  only slows the outer iteration; the answer is the FP64 operator's;
* ``ilu_preconditioner(nearfield)`` -- an incomplete LU of the nearfield
  matrix as a right preconditioner for both (the reference's
  acceptance_tests/ilu_preconditioning.py:12-31 factors the nearfield with
  scipy's spilu for its GMRES).
"""
import math

import numpy as np


def _dot(a, b):
    return float((a * b).sum())


def _norm(a):
    return math.sqrt(_dot(a, a))


def gmres(matvec, b, x0=None, restart=50, tol=1e-10, maxiter=1000, callback=None, precond=None):
    """Restarted GMRES(restart).  Returns (x, info, iterations); info = 0 on
    convergence (||b - A x|| <= tol ||b||), 1 otherwise.  precond: an
    approximate inverse M (callable), applied on the right: GMRES runs on
    A M and x = M y, so the residuals it reports are the true ones."""
    M = precond if precond is not None else (lambda v: v)
    x = b * 0 if x0 is None else x0.copy() if hasattr(x0, "copy") else x0.clone()
    bnorm = _norm(b)
    if bnorm == 0.0:
        return x, 0, 0
    it = 0
    while it < maxiter:
        r = b - matvec(x)
        beta = _norm(r)
        if beta <= tol * bnorm:
            return x, 0, it
        V = [r / beta]
        H = np.zeros((restart + 1, restart))
        cs = np.zeros(restart)
        sn = np.zeros(restart)
        g = np.zeros(restart + 1)
        g[0] = beta
        k_done = 0
        for k in range(restart):
            w = matvec(M(V[k]))
            for j in range(k + 1):
                H[j, k] = _dot(w, V[j])
                w = w - H[j, k] * V[j]
            H[k + 1, k] = _norm(w)
            V.append(w / H[k + 1, k] if H[k + 1, k] > 0 else w)
            for j in range(k):
                t = cs[j] * H[j, k] + sn[j] * H[j + 1, k]
                H[j + 1, k] = -sn[j] * H[j, k] + cs[j] * H[j + 1, k]
                H[j, k] = t
            den = math.hypot(H[k, k], H[k + 1, k])
            cs[k], sn[k] = (1.0, 0.0) if den == 0 else (H[k, k] / den, H[k + 1, k] / den)
            H[k, k] = cs[k] * H[k, k] + sn[k] * H[k + 1, k]
            H[k + 1, k] = 0.0
            g[k + 1] = -sn[k] * g[k]
            g[k] = cs[k] * g[k]
            it += 1
            k_done = k + 1
            if callback:
                callback(abs(g[k + 1]) / bnorm)
            if abs(g[k + 1]) <= tol * bnorm or it >= maxiter:
                break
        y = np.linalg.solve(np.triu(H[:k_done, :k_done]), g[:k_done])
        z = y[0] * V[0]
        for j in range(1, k_done):
            z = z + y[j] * V[j]
        x = x + M(z)
    r = b - matvec(x)
    return x, 0 if _norm(r) <= tol * bnorm else 1, it


def refined_solve(apply_fp64, apply_fast, b, tol=1e-10, inner_tol=1e-6, restart=50,
                  max_outer=20, inner_maxiter=500, precond=None):
    """FP64 iterative refinement.  Returns (x, history) where history holds
    (outer iteration, inner iterations, relative FP64 residual).  precond is
    handed to the inner GMRES (right preconditioning)."""
    x = b * 0
    bnorm = _norm(b)
    history = []
    r = b - apply_fp64(x)
    for outer in range(max_outer):
        rel = _norm(r) / bnorm
        if rel <= tol:
            history.append((outer, 0, rel))
            break
        d, _, its = gmres(apply_fast, r, restart=restart, tol=inner_tol, maxiter=inner_maxiter,
                          precond=precond)
        x = x + d
        r = b - apply_fp64(x)
        history.append((outer, its, _norm(r) / bnorm))
    return x, history


def exterior_dirichlet_system(single, double):
    """The exterior Laplace Dirichlet problem as a second-kind system.

    The field outside a closed surface is represented by a combined layer,
    u = D_std mu + S mu (D_std the standard double layer, with kernel
    dG/dn_y, G = 1 / (4 pi r)); its exterior limit on the surface gives
    (1/2 I + K + S) mu = g, uniquely solvable for every Dirichlet datum g
    (the single layer carries the field's monopole, which a double layer
    cannot).  The library's LaplaceDouble kernel is n_y . (y - x) / (4 pi r^3)
    = -dG/dn_y, so with its operators D and S the system reads
    (1/2 I - D + S) mu = g, and the field u = -D mu + S mu.  single, double:
    callables applying S and D (any precision form).  Returns the system's
    apply."""
    return lambda v: 0.5 * v - double(v) + single(v)


def ilu_preconditioner(nearfield, drop_tol=1e-4, fill_factor=10.0):
    """Incomplete LU of a nearfield matrix as an approximate inverse.

    nearfield: a tbempy SparseOperator (its CSR arrays are read back), a scipy
    sparse matrix, or a dense array.  Returns M(v) that solves L U z = v on
    the host with scipy's spilu (the reference's choice); numpy vectors or
    torch tensors (copied to the host and back), one or several right-hand
    sides ([n] or [n_rhs, n])."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    if hasattr(nearfield, "row_ptrs"):
        A = sp.csr_matrix((nearfield.values(), nearfield.column_indices(), nearfield.row_ptrs()),
                          shape=(nearfield.n_rows(), nearfield.n_cols()))
    else:
        A = sp.csr_matrix(nearfield)
    lu = spla.spilu(A.tocsc(), drop_tol=drop_tol, fill_factor=fill_factor)

    def apply(v):
        if hasattr(v, "detach"):  # torch
            import torch
            h = v.detach().cpu().numpy()
            out = np.stack([lu.solve(r) for r in h]) if h.ndim == 2 else lu.solve(h)
            return torch.as_tensor(out, dtype=v.dtype, device=v.device)
        return np.stack([lu.solve(r) for r in v]) if v.ndim == 2 else lu.solve(v)

    return apply

