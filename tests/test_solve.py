"""CPU tests of the solver driver: restarted GMRES and FP64 iterative
refinement around a less accurate inner operator (host logic only)."""
import numpy as np

from tbempy import solve


def test_gmres_solves_well_conditioned_system():
    rng = np.random.default_rng(0)
    n = 200
    A = np.eye(n) * 2 + rng.normal(size=(n, n)) / (4 * np.sqrt(n))
    b = rng.normal(size=n)
    x, info, its = solve.gmres(lambda v: A @ v, b, restart=30, tol=1e-12, maxiter=500)
    assert info == 0
    assert np.linalg.norm(A @ x - b) <= 1e-11 * np.linalg.norm(b)


def test_gmres_restart_and_zero_rhs():
    rng = np.random.default_rng(1)
    n = 120
    A = np.eye(n) + 0.5 * rng.normal(size=(n, n)) / np.sqrt(n)
    b = rng.normal(size=n)
    x, info, its = solve.gmres(lambda v: A @ v, b, restart=5, tol=1e-10, maxiter=2000)
    assert info == 0 and its > 5
    x0, info0, _ = solve.gmres(lambda v: A @ v, np.zeros(n))
    assert info0 == 0 and not x0.any()


def test_refinement_reaches_fp64_accuracy_with_a_perturbed_inner_operator():
    rng = np.random.default_rng(2)
    n = 300
    A = np.eye(n) * 0.5 + rng.normal(size=(n, n)) / (3 * np.sqrt(n))
    E = rng.normal(size=(n, n)) * 1e-6 / np.sqrt(n)   # the "mixed precision" error
    b = rng.normal(size=n)
    x, hist = solve.refined_solve(lambda v: A @ v, lambda v: (A + E) @ v, b, tol=1e-12,
                                  inner_tol=1e-6)
    assert hist[-1][2] <= 1e-12
    assert np.linalg.norm(A @ x - b) <= 1e-12 * np.linalg.norm(b)
    assert len(hist) <= 6


def test_right_preconditioning_with_the_exact_inverse_converges_at_once():
    rng = np.random.default_rng(3)
    n = 150
    A = np.eye(n) + rng.normal(size=(n, n)) / np.sqrt(n)
    b = rng.normal(size=n)
    Ainv = np.linalg.inv(A)
    x, info, its = solve.gmres(lambda v: A @ v, b, tol=1e-12, precond=lambda v: Ainv @ v)
    assert info == 0 and its <= 2
    assert np.linalg.norm(A @ x - b) <= 1e-11 * np.linalg.norm(b)


def test_nearfield_ilu_cuts_gmres_iterations():
    """A = N + F with a strong sparse nearfield N and a weak dense farfield F:
    the ILU of N as right preconditioner (the reference's acceptance setup)
    reaches the same solution in far fewer iterations, also inside the FP64
    refinement."""
    import scipy.sparse as sp
    rng = np.random.default_rng(4)
    n = 400
    N = sp.random(n, n, density=0.02, random_state=5, format="csr") * 3.0
    N = N + sp.diags(np.linspace(1.0, 50.0, n))
    F = rng.normal(size=(n, n)) * 0.05 / np.sqrt(n)
    A = N.toarray() + F
    b = rng.normal(size=n)
    mv = lambda v: A @ v
    x0, info0, it0 = solve.gmres(mv, b, restart=30, tol=1e-10, maxiter=3000)
    M = solve.ilu_preconditioner(N)
    x1, info1, it1 = solve.gmres(mv, b, restart=30, tol=1e-10, maxiter=3000, precond=M)
    assert info0 == 0 and info1 == 0
    assert it1 * 4 <= it0, (it0, it1)
    assert np.linalg.norm(x1 - x0) <= 1e-8 * np.linalg.norm(x0)
    E = rng.normal(size=(n, n)) * 1e-6 / np.sqrt(n)
    x2, hist = solve.refined_solve(mv, lambda v: (A + E) @ v, b, tol=1e-12, precond=M)
    assert np.linalg.norm(A @ x2 - b) <= 1e-12 * np.linalg.norm(b)
    # several right-hand sides at once through the preconditioner
    V = rng.normal(size=(2, n))
    W = M(V)
    assert W.shape == V.shape and np.allclose(W[1], M(V[1]))

