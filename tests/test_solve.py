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
